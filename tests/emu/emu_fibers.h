// Fiber-based SIMT launcher for the CPU emulation of the engine's kernels (tests only):
// the threads of a CTA are ucontext fibers of one host thread; each runs until its next
// __syncthreads, and the barrier opens once every fiber has arrived or returned.  CTAs
// run one after another.  Include once per harness, before the kernel sources.
#pragma once
#include <ucontext.h>

#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "cuda_runtime.h"

uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim, gridDim;

namespace {
struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  int state = 0;   // 0 runnable, 1 at the barrier, 2 returned
};
ucontext_t g_sched;
std::vector<Fiber> g_fib;
int g_cur = 0;
const std::function<void()>* g_body = nullptr;
void fiber_main() {
  (*g_body)();
  g_fib[g_cur].state = 2;
  swapcontext(&g_fib[g_cur].ctx, &g_sched);
}
}  // namespace

void emu_syncthreads() {
  g_fib[g_cur].state = 1;
  swapcontext(&g_fib[g_cur].ctx, &g_sched);
}
static std::vector<double> g_dyn;   // dynamic shared memory of the running CTA
template <class T>
T* emu_dyn_smem() { return reinterpret_cast<T*>(g_dyn.data()); }
inline int atomicMax(int* p, int v) {
  const int o = *p;
  if (v > o) *p = v;
  return o;
}
inline double atomicAdd(double* p, double v) {
  const double o = *p;
  *p += v;
  return o;
}

namespace {

// grid CTAs of `block` fibers with dyn_bytes of dynamic shared memory
template <class F>
void launch(int grid, int block, size_t dyn_bytes, F&& f) {
  const std::function<void()> body(f);
  g_body = &body;
  blockDim = dim3{(unsigned)block, 1, 1};
  gridDim = dim3{(unsigned)grid, 1, 1};
  if ((int)g_fib.size() < block) g_fib.resize(block);
  for (int b = 0; b < grid; ++b) {
    blockIdx = uint3{(unsigned)b, 0, 0};
    g_dyn.assign(dyn_bytes / 8 + 1, 0.0);
    for (int t = 0; t < block; ++t) {
      Fiber& fb = g_fib[t];
      if (fb.stack.empty()) fb.stack.resize(1 << 17);
      getcontext(&fb.ctx);
      fb.ctx.uc_stack.ss_sp = fb.stack.data();
      fb.ctx.uc_stack.ss_size = fb.stack.size();
      fb.ctx.uc_link = nullptr;
      makecontext(&fb.ctx, fiber_main, 0);
      fb.state = 0;
    }
    for (;;) {
      // run every runnable thread up to its next barrier (or its return)
      for (int t = 0; t < block; ++t) {
        if (g_fib[t].state != 0) continue;
        g_cur = t;
        threadIdx = uint3{(unsigned)t, 0, 0};
        swapcontext(&g_sched, &g_fib[t].ctx);
      }
      bool any = false;
      for (int t = 0; t < block; ++t)
        if (g_fib[t].state == 1) {
          g_fib[t].state = 0;
          any = true;
        }
      if (!any) break;
    }
  }
}

}  // namespace

