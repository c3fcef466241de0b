/* Host-emulation stand-in for thrust::inner_product: a sequential FP64 sum in
 * index order (the reference's library reduction differs only in order). */
#ifndef EMU_THRUST_INNER_PRODUCT_H
#define EMU_THRUST_INNER_PRODUCT_H
#include "device_ptr.h"
namespace thrust {
template <typename T, typename V>
V inner_product(device_ptr<T> a, device_ptr<T> a_end, device_ptr<T> b, V init) {
  V s = init;
  for (T *x = a.p, *y = b.p; x != a_end.p; ++x, ++y) s += (*x) * (*y);
  return s;
}
}  // namespace thrust
#endif
