/* Host-emulation stand-in for thrust::device_ptr over host memory. */
#ifndef EMU_THRUST_DEVICE_PTR_H
#define EMU_THRUST_DEVICE_PTR_H
#include <stddef.h>
namespace thrust {
template <typename T>
struct device_ptr {
  T *p;
  explicit device_ptr(T *q) : p(q) {}
  device_ptr operator+(ptrdiff_t n) const { return device_ptr(p + n); }
};
}  // namespace thrust
#endif
