// SIMT emulation of the symmetry-adapted kernels (k_sitesym.cu) on the host, for the CPU
// tests: every CTA runs as blockDim.x host threads with a barrier for __syncthreads,
// one CTA after another.  The kernel source is compiled unchanged against the stand-in
// <cuda_runtime.h> beside this file.  Entry points take flat host arrays (ctypes).
#include <barrier>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "cuda_runtime.h"

thread_local uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim, gridDim;
static std::barrier<>* g_bar = nullptr;
void emu_syncthreads() { g_bar->arrive_and_wait(); }

#include "k_sitesym.cu"
#include "sym_tables.h"

namespace {

// grid CTAs of `block` threads; only >= 0 runs that one CTA alone
template <class F>
void emu_launch(int grid, int block, F&& body, int only = -1) {
  blockDim = dim3{(unsigned)block, 1, 1};
  gridDim = dim3{(unsigned)grid, 1, 1};
  for (int b = 0; b < grid; ++b) {
    if (only >= 0 && b != only) continue;
    blockIdx = uint3{(unsigned)b, 0, 0};
    std::barrier<> bar(block);
    g_bar = &bar;
    std::vector<std::thread> th;
    th.reserve(block);
    for (int t = 0; t < block; ++t)
      th.emplace_back([&, t] {
        threadIdx = uint3{(unsigned)t, 0, 0};
        body();
        g_bar->arrive_and_drop();
      });
    for (auto& x : th) x.join();
  }
}

struct Emu {
  w90g::SymTables t;
  std::vector<int> ints;
  std::vector<double> work;
  w90g::CtrlState st{};
  w90g::Problem P{};
  int offs[2] = {0, 0};
  w90g::WorkMap wm{};
};

// the engine's layout of the tables (Engine::set_sym)
int setup(Emu& e, int W, int K, int nsym, int nkirr, const int* ik2ir, const int* ir2ik, const int* kptsym,
          const double* dw, const double* db) {
  std::string msg;
  if (int rc = w90g::build_sym_tables(W, W, nsym, nkirr, K, ik2ir, ir2ik, kptsym, dw, db, e.t, msg)) return rc;
  auto& t = e.t;
  e.ints.clear();
  for (auto* v : {&t.ik, &t.moff, &t.mem, &t.goff, &t.grp}) e.ints.insert(e.ints.end(), v->begin(), v->end());
  e.ints.insert(e.ints.end(), (size_t)t.nir, -7);
  int* base = e.ints.data();
  size_t o = 0;
  e.P.W = W;
  e.P.K = K;
  e.P.sym_nir = t.nir;
  e.P.sym_ik = base;
  e.P.sym_moff = base + (o += t.ik.size());
  e.P.sym_mem = base + (o += t.moff.size());
  e.P.sym_goff = base + (o += t.mem.size());
  e.P.sym_grp = base + (o += t.goff.size());
  e.P.sym_status = base + (o += t.grp.size());
  e.P.sym_d = reinterpret_cast<const double2*>(t.d.data());
  e.P.sym_db = reinterpret_cast<const double2*>(t.db.data());
  e.work.assign((size_t)t.nir * w90g::kSymWork * W * W * 2, 0.0);
  e.P.sym_work = reinterpret_cast<double2*>(e.work.data());
  e.P.st = &e.st;
  e.offs[1] = t.nir;
  e.wm = w90g::WorkMap{e.offs, 1};
  return 0;
}

}  // namespace

extern "C" {

// gradient symmetrisation: G (K, W, W) column-major blocks, in place; Dprev likewise;
// gpart (K * ntt * 2), ntt = ceil(W/32)^2.  Returns 0 or the table builder's code.
int emu_sym_grad(int W, int K, int nsym, int nkirr, const int* ik2ir, const int* ir2ik, const int* kptsym,
                 const double* dw, const double* db, double* G, double* Dprev, double* gpart) {
  Emu e;
  if (int rc = setup(e, W, K, nsym, nkirr, ik2ir, ir2ik, kptsym, dw, db)) return rc;
  e.P.G = reinterpret_cast<double2*>(G);
  e.P.D = reinterpret_cast<double2*>(Dprev);
  e.P.gpart = gpart;
  emu_launch(e.t.nir, 256, [&] { w90g::k_sym_grad(&e.P, e.wm); });
  return 0;
}

// search direction: D = cg G + cd Dprev at the irreducible k, rotated onto the stars (D in place)
int emu_sym_dir(int W, int K, int nsym, int nkirr, const int* ik2ir, const int* ir2ik, const int* kptsym,
                const double* dw, const double* db, double* G, double* D, double cg, double cd) {
  Emu e;
  if (int rc = setup(e, W, K, nsym, nkirr, ik2ir, ir2ik, kptsym, dw, db)) return rc;
  e.P.G = reinterpret_cast<double2*>(G);
  e.P.D = reinterpret_cast<double2*>(D);
  e.st.coefG = cg;
  e.st.coefD = cd;
  emu_launch(e.t.nir, 256, [&] { w90g::k_sym_dir(&e.P, e.wm); });
  return 0;
}

// symmetry-adapted U (K, W, W) in place; status[nkirr] out; threads per CTA (a power of
// two <= 256; the engine launches 256) and only >= 0 to run one CTA alone
int emu_sym_u(int W, int K, int nsym, int nkirr, const int* ik2ir, const int* ir2ik, const int* kptsym,
              const double* dw, const double* db, double eps, double* U, int* status, int threads, int only) {
  Emu e;
  if (int rc = setup(e, W, K, nsym, nkirr, ik2ir, ir2ik, kptsym, dw, db)) return rc;
  e.P.U[0] = reinterpret_cast<double2*>(U);
  e.P.sym_eps = eps;
  emu_launch(e.t.nir, threads, [&] { w90g::k_sym_u(&e.P, e.wm); }, only);
  std::memcpy(status, e.P.sym_status, sizeof(int) * e.t.nir);
  return 0;
}

}  // extern "C"
