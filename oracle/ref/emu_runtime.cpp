// emu_runtime.cpp -- fiber scheduler behind emu_cuda.h (test infrastructure).
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "shim/emu_cuda.h"

namespace emu {
uint3 cur_tid, cur_bid;
dim3 cur_bdim, cur_gdim;

namespace {
const size_t kStack = 128 * 1024;
struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  uint3 tid;
  bool done = false;
};
ucontext_t g_sched;
std::vector<Fiber> g_fibers;
const std::function<void()> *g_body = nullptr;
int g_cur = -1;

void trampoline() {
  (*g_body)();
  g_fibers[g_cur].done = true;
  // returning switches to uc_link (the scheduler)
}
}  // namespace

void sync() {
  if (g_cur < 0) {
    fprintf(stderr, "emu: __syncthreads outside a kernel\n");
    abort();
  }
  swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

void launch(dim3 grid, dim3 block, const std::function<void()> &body) {
  const int nt = (int)(block.x * block.y * block.z);
  if (nt <= 0 || grid.x * grid.y * grid.z == 0) return;
  if ((int)g_fibers.size() < nt) g_fibers.resize(nt);
  for (auto &f : g_fibers)
    if (f.stack.size() < kStack) f.stack.resize(kStack);
  const std::function<void()> *saved = g_body;
  g_body = &body;
  cur_bdim = block;
  cur_gdim = grid;
  for (unsigned bz = 0; bz < grid.z; bz++)
    for (unsigned by = 0; by < grid.y; by++)
      for (unsigned bx = 0; bx < grid.x; bx++) {
        cur_bid = uint3{bx, by, bz};
        for (int t = 0; t < nt; t++) {
          Fiber &f = g_fibers[t];
          f.tid = uint3{(unsigned)(t % block.x), (unsigned)((t / block.x) % block.y),
                        (unsigned)(t / (block.x * block.y))};
          f.done = false;
          getcontext(&f.ctx);
          f.ctx.uc_stack.ss_sp = f.stack.data();
          f.ctx.uc_stack.ss_size = f.stack.size();
          f.ctx.uc_link = &g_sched;
          makecontext(&f.ctx, trampoline, 0);
        }
        int alive = nt;
        while (alive > 0) {
          alive = 0;
          for (int t = 0; t < nt; t++) {
            Fiber &f = g_fibers[t];
            if (f.done) continue;
            g_cur = t;
            cur_tid = f.tid;
            swapcontext(&g_sched, &f.ctx);
            if (!f.done) alive++;
          }
        }
        g_cur = -1;
      }
  g_body = saved;
}
}  // namespace emu
