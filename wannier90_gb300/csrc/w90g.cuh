// Shared device-side definitions of the GB300 MLWF engine.
//
// Layout in HBM (one "problem" = one wann_main solve):
//   M[buf][k][b]  W x W complex128 block, column-major (element (m,n) at n*W+m),
//                 exactly the reference's m_matrix_loc(W,W,B,K) layout.
//   U[buf][k]     W x W complex128, column-major (u_matrix(W,W,K)).
//   G[k], D[k]    gradient (cdodq) and kept search direction (cdqkeep).
//   dU[k]         the rotation exp(s*D(k)) of the current step.
//   diag_ln, diag_abs2 [k][b][n], offd [k][b]  per-block statistics written by the
//                 M-update epilogue and read by the spread reduction.
// Two buffers of M and U are kept: `st->cur` selects the accepted state; every update
// reads buffer cur and writes buffer cur^1, so the line-search "restore" of the
// reference (src/wannierise.F90:608-615, :668-675) never copies memory.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace w90g {

// ----------------------------------------------------------------------------
// complex helpers (double2 = re, im)
// ----------------------------------------------------------------------------
__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return cmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return cmk(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return cmk(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__host__ __device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return cmk(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
#ifdef __CUDACC__
// acc += a * b
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
__device__ __forceinline__ void cfmac(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // plain a*conj(b)/|b|^2, as Fortran complex division of well-scaled operands
  double d = b.x * b.x + b.y * b.y;
  double2 n = cmulc(a, b);
  return cmk(n.x / d, n.y / d);
}
#endif

// ----------------------------------------------------------------------------
// controller state of one problem (device memory, one per problem)
// Mirrors the scalar locals of wann_main (src/wannierise.F90:150-175).
// ----------------------------------------------------------------------------
constexpr int kMaxConvWindow = 64;

// With selective localisation om_i is not computed (0), om_od holds
// Omega_IOD + Omega_nu (the sum the reference prints as O_IOD) and om_nu the centre
// constraint's Omega_nu (0 otherwise).
struct Spread {
  double om_i, om_d, om_od, om_tot, om_nu;
};

struct CtrlState {
  // loop bookkeeping
  int iter;            // iterations completed
  int done;            // 1 => no further work (converged, num_iter reached or error)
  int cur;             // accepted buffer index (0/1)
  int error;           // 0 ok, >0 engine error code
  int ncg;
  int lquad;
  int do_second;       // second update (parabolic optimum) required this iteration
  int conv_count, noise_count, lrandom, lfirst, lconverged;
  int first_pass;
  int use_gp;          // precond: the search direction starts from the preconditioned gradient
  int irguide;         // guiding centres: 0 until the first wann_phases call
  // CG
  double gcnorm0, gcnorm1, gcfac, doda0;
  double coefG, coefD;   // D <- coefG*G + coefD*D_prev
  double s_trial;        // X = s*D for the trial step
  double s_second;       // X = s*D for the optimal step
  double alphamin, falphamin;
  double save_spread;
  double om_invariant;
  Spread wann, old, slot[2];   // slot[0] = trial spread, slot[1] = optimal-step spread
  double history[kMaxConvWindow];
  double exp_products;   // W^3 complex products spent in exp(s D) and U dU (work counter)
  // spread passes: CTAs of k_omega_p1 / k_omega_p2 that have finished this launch (the
  // last one reduces the chunk partials and sets the count back to 0), and the Omega_OD,
  // Omega_I chunk totals that pass 1's last CTA hands to pass 2's
  unsigned omega_arrive[2];
  double omega_tot[2];
};

// wann_control_type subset used on device (src/wannier90_types.F90:170-192)
struct Control {
  int num_iter, num_cg_steps, conv_window, conv_noise_num;
  int lfixstep, pad;
  double conv_tol, trial_step, fixed_step, conv_noise_amp;
};

// per-iteration record (the <-- CONV / <-- SPRD lines, src/wannierise.F90:704-756)
constexpr int kLogStride = 10;  // iter, delta, rms_grad, om_tot, om_d, om_od, lquad, alphamin, t_ns, om_nu

struct Problem {
  int W, K, B, nthr_pad;
  double wbtot;
  double2* M[2];
  double2* U[2];
  double2* G;
  double2* D;
  double2* dU;
  double2* work;        // exp / eig workspace (W > 32): 6*W*W per k
  double2* tbuf;        // M-update intermediate (W > 32): W*W per (k,b)
  const int* nnlist;    // [k][b] 0-based
  const double* bk;     // [k][b][3]
  const double* wb;     // [b]
  double* diag_ln;      // [k][b][n]  Im ln M_nn
  double* diag_abs2;    // [k][b][n]  |M_nn|^2
  double* offd;         // [k][b]     sum_{m!=n} |M_mn|^2
  double* gpart;        // [k][2]     sum |G|^2, sum Re conj(G) D_prev  (per k)
  double* centres;      // [slot][4][W]: rave(3,W) + r2ave-rave2 (W) per spread slot; slot 2 = accepted
  double* log;          // [num_iter+1][kLogStride]
  double* log_centres;  // [num_iter+1][4][W]
  double2* M0;          // tensor path: M at entry (never modified)
  unsigned char* m0s;   // tensor path: step 1's A operand (M0 rows) in BF16 digit planes,
                        // the shared-memory image of every (k, tile, K chunk)
  int* m0s_exp;         // tensor path: the row exponents of those tiles [k][tile][128]
  int* zexp;            // pipelined tensor path: step 2's row exponents [k][b][row of Z(k,b)],
                        // written by step 1's epilogue
  unsigned char* ub2;   // pipelined tensor path: step 2's B operand -- the digit planes of U(k)
                        // in the shared-memory layout, per k -- written by step 1's B producer
  int* ub2_exp;         // ... and the column exponents of U(k) [k][WP]
  double2* U0;          // tensor path: U at entry; U[] then holds R = U0^H U
  const int* inv_nnlist;  // tensor path: [k'][i] = k*B+b with nnlist(k,b) = k'
  double* frob0;        // tensor path: |M0(k,b)|_F^2
  double* opart1;       // [nchunk][4W+2] spread partials (pass 1)
  double* opart2;       // [nchunk]       Omega_D partials (pass 2)
  int nchunk;           // ceil(K*B / 64)
  int tensor;           // 1: M update on tensor cores (tcgen05, exact BF16 slicing)
  CtrlState* st;
  Control ctl;
  int max_exp_squarings;
  int precond;          // 1: precond_search_direction (src/wannierise.F90:1256-1368)
  int nrpts;            // Wigner-Seitz points of the preconditioner
  int pad3;
  const double2* pc_kr;   // [k][r] exp(-i 2 pi k.R_r)
  const double* pc_r2;    // [r] |R_r|^2 as the reference forms it
  const double* pc_ndeg;  // [r] degeneracy of R_r
  double2* pc_gr;         // [r][W*W] gradient in real space
  double2* pc_gp;         // [k][W*W] preconditioned gradient
  double* pc_part;        // [tile] Re <Gp, G> partials of the back transform
  // guiding centres (wann_phases, src/wannierise.F90:1756-1976); sheet == null: off
  int guiding, nnh, no_guide_iter, guide_cycles;
  const double* bka;      // [nnh][3] b directions
  const int* neigh;       // [k][nnh] neighbour index of each direction
  double* rguide;         // [3][W] guiding centres (Cartesian, Angstrom)
  double* sheet;          // [k][b][n] branch offsets b . rguide_n
  double2* csheet;        // [k][b][n] exp(i sheet)
  // selective localisation (src/wannierise.F90:2144-2211, :2431-2509): slwf_num > 0 makes
  // WFs 0..slwf_num-1 the objective ones; slwf_lambda is lambda_loc (0 unless the centres
  // are constrained); slwf_c [3][W] the constrained centres (Cartesian, Angstrom), zero
  // when unconstrained; slwf_nu0 = lambda * sum_{n < slwf_num} |c_n|^2
  int slwf_num, pad4;
  double slwf_lambda, slwf_nu0;
  const double* slwf_c;
  // symmetry-adapted mode (site_symmetry = T, src/sitesym.F90): sym_nir > 0 irreducible
  // k-points; per irreducible ir its k (sym_ik), its star's reducible members
  // sym_mem[sym_moff[ir] .. sym_moff[ir+1]) as (k, slot) pairs in the reference's
  // first-occurrence order, its little group {R : R k = k} sym_grp[sym_goff[ir] ..
  // sym_goff[ir+1]) as (isym, slot) pairs in isym order (isym 0-based, the identity
  // first); slot s indexes D(R, k_ir) = sym_d[s] and d(R, k_ir) = sym_db[s] (W x W,
  // column-major); sym_work kSymWork W x W matrices per irreducible k; sym_status the
  // initial symmetrisation's result per irreducible k
  int sym_nir, pad5;
  double sym_eps;
  const int* sym_ik;
  const int* sym_moff;
  const int* sym_mem;
  const int* sym_goff;
  const int* sym_grp;
  const double2* sym_d;
  const double2* sym_db;
  double2* sym_work;
  int* sym_status;
};

constexpr int kSymWork = 5;

// Work map: blockIdx.x -> (problem, local index) over a prefix sum.
struct WorkMap {
  const int* offs;  // nprob+1 prefix sums of work items per problem
  int nprob;
};

#ifdef __CUDACC__
// Im ln M_nn(k,b) on the branch of the guiding centres: aimag(log(csheet*M_nn)) - sheet
// (src/wannierise.F90:2036-2041, :2368-2374); kbn = (k*B + b)*W + n
__device__ __forceinline__ double guided_ln(const Problem& P, size_t kbn, double2 d) {
  if (!P.sheet) return atan2(d.y, d.x);
  const double2 c = P.csheet[kbn];
  const double2 z = cmul(c, d);
  return atan2(z.y, z.x) - P.sheet[kbn];
}

__device__ __forceinline__ int locate(const WorkMap& wm, int item, int& local) {
  int lo = 0, hi = wm.nprob - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(wm.offs + mid) <= item) lo = mid; else hi = mid - 1;
  }
  local = item - __ldg(wm.offs + lo);
  return lo;
}
#endif

// Host: one strided copy of the top-left W x W of each of nblk complex128 blocks
// (leading dimensions ldd / lds), e.g. the num_wann x num_wann part of the
// (num_bands, num_bands) blocks of m_matrix_local.
inline cudaError_t copy_wblocks(void* dst, int ldd, const void* src, int lds, int W, int nblk, cudaMemcpyKind kind,
                                cudaStream_t st) {
  cudaMemcpy3DParms q = {};
  q.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), (size_t)lds * 16, (size_t)W * 16, (size_t)lds);
  q.dstPtr = make_cudaPitchedPtr(dst, (size_t)ldd * 16, (size_t)W * 16, (size_t)ldd);
  q.extent = make_cudaExtent((size_t)W * 16, (size_t)W, (size_t)nblk);
  q.kind = kind;
  return cudaMemcpy3DAsync(&q, st);
}

}  // namespace w90g
