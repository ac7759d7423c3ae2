// Disentanglement on the GPU: dis_main (src/disentangle.F90:31-284) for the k-point path
// without site symmetry, plus the rotation of setup_m_loc (:286-370), as called by the
// library's w90_disentangle (src/library_interface.F90:362-420).
//
// The windows (dis_windows, :851-1171) are set up on the host; everything per k-point runs
// as one CTA per k in FP64: the projection onto the outer window (dis_project), the
// completion of the frozen states (dis_proj_froz), every iteration of the Omega_I
// minimisation (internal_zmatrix, mixing, diagonalisation, Omega_I; dis_extract), the
// subspace-Hamiltonian gauge, and the final rotations (M_opt, internal_find_u,
// setup_m_loc).  Hermitian eigenproblems use the CTA Jacobi solver (eigenvalues sorted
// ascending, as ZHPEVX returns them); the SVD-based polar factors of the reference
// (Z V^dagger) are computed as X (X^H X)^{-1/2}, the same matrix for full-rank X.  The
// host reads back two numbers per k and iteration for the convergence test
// (internal_test_convergence, :2866-2920).
//
// Layout (column-major, as the reference's arrays): M[k][b] nb x nb, A / U_opt [k] nb x W,
// Z [k] nb x nb, a per-k workspace of kWs nb^2 complex entries in global memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "cta.cuh"
#include "dis.h"

namespace w90g {

namespace {

constexpr int kWs = 8;   // workspace per k, in units of nb*nb complex entries
// dynamic shared memory of k_dis_step (3 m x m) and k_dis_rotate (W x nb + 2 W x W) at
// the largest band count (64)
constexpr size_t kDisMaxSmem = 3 * 64 * 64 * 16;

struct DisDev {
  int nb, W, K, B;
  double wbtot, mix;
  const int* nnlist;     // [k][b]
  const double* wb;      // [b]
  const int* ndim;       // [k] outer-window states
  const int* nfirst;     // [k] first band of the window (0-based)
  const int* nfroz;      // [k] frozen states
  const int* ffirst;     // [k] first frozen state inside the window (0-based)
  const int* nfidx;      // [k][nb] non-frozen window states (0-based)
  const double* eig;     // [k][nb] window eigenvalues (shifted to the window)
  const double2* Mraw;   // [k][b] nb x nb, the caller's overlaps
  double2* Mw;           // [k][b] nb x nb, window block at the top left
  double2* A;            // [k] nb x W windowed projections
  double2* U[2];         // [k] nb x W, U_opt (double buffered over the iterations)
  double2* Zin;          // [k] nb x nb
  double2* Zout;         // [k] nb x nb
  double2* U0;           // [k] W x W  (internal_find_u)
  double2* M0;           // [k][b] W x W, the rotated overlaps for wann_main
  double2* ws;           // [k] kWs nb^2
  double* wk1;           // [k] Omega_I(i-1) parts (from the eigenvalues)
  double* wk;            // [k] Omega_I(i) parts (from the overlaps)
  int* status;           // [k]
  double2* Vz;           // [k] m x m eigenvectors of the last Z (warm start of the next)
  int* max_sweeps;       // Jacobi sweeps, max over k and iterations
  // symmetry-adapted mode (sym_nir > 0 irreducible k): the star / little-group tables of
  // the wannierisation (Problem::sym_*), the band representation d(R,k) as nb x nb slots
  // (sym_db) and the Wannier one D(R,k) as W x W slots (sym_d); sym_ws kDisSymWs nb x nb
  // matrices per irreducible k; sym_status per irreducible k
  int sym_nir, sym_nsym;
  double sym_eps;
  const int* sym_ik;
  const int* sym_moff;
  const int* sym_mem;
  const int* sym_goff;
  const int* sym_grp;
  const double2* sym_d;
  const double2* sym_db;
  double2* sym_ws;
  int* sym_status;
};

constexpr int kDisSymWs = 16;

__device__ __forceinline__ double2 op_el(const double2* X, int ld, bool c, int i, int j) {
  // element (i, j) of X (c = false) or of X^H (c = true)
  return c ? cconj(X[(size_t)i * ld + j]) : X[(size_t)j * ld + i];
}

// C (m x n, ldc) = op(A) op(B) with inner dimension kk (C must not alias A or B)
__device__ void cta_zgemm(double2* C, int ldc, const double2* A, int lda, bool ca, const double2* B, int ldb,
                          bool cb, int m, int n, int kk) {
  for (int e = threadIdx.x; e < m * n; e += blockDim.x) {
    const int i = e % m, j = e / m;
    double2 acc = cmk(0, 0);
    for (int l = 0; l < kk; ++l) cfma(acc, op_el(A, lda, ca, i, l), op_el(B, ldb, cb, l, j));
    C[(size_t)j * ldc + i] = acc;
  }
}

struct JacobiScratch {
  double* red;
  double* rc;
  double2* rse;
  int* rp;
  int* rq;
};

// ascending order of the Jacobi eigenvalues (diagonal of H, n x n) into ord[0..n), ev[]
__device__ void sort_eigs(const double2* H, int n, int* ord, double* ev) {
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      ev[i] = H[(size_t)i * n + i].x;
      ord[i] = i;
    }
    for (int i = 1; i < n; ++i) {
      const int o = ord[i];
      const double v = ev[o];
      int j = i - 1;
      while (j >= 0 && ev[ord[j]] > v) {
        ord[j + 1] = ord[j];
        --j;
      }
      ord[j + 1] = o;
    }
  }
  __syncthreads();
}

// Q (m x w, ldq) = X (X^H X)^{-1/2}; scratch S, V, T (w x w) and Y (m x w).  Sets *flag
// to 0, or 1 for a rank-deficient X, 2 when the eigensolver did not converge.
__device__ void cta_polar(double2* Q, int ldq, const double2* X, int ldx, int m, int w, double2* S, double2* V,
                          double2* T, double2* Y, JacobiScratch js, int* flag) {
  cta_zgemm(S, w, X, ldx, true, X, ldx, false, w, w, m);
  __syncthreads();
  const int sw = cta_jacobi(S, V, w, 60, js.red, js.rc, js.rse, js.rp, js.rq);
  if (threadIdx.x == 0) *flag = (sw < 0) ? 2 : 0;
  __syncthreads();
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int j = e / w;
    const double l = S[(size_t)j * w + j].x;
    if (!(l > 0.0)) *flag = 1;
    T[e] = cscale(V[e], 1.0 / sqrt(fmax(l, 1e-300)));
  }
  __syncthreads();
  cta_zgemm(Y, m, X, ldx, false, T, w, false, m, w, w);
  __syncthreads();
  cta_zgemm(Q, ldq, Y, m, false, V, w, true, m, w, w);
  __syncthreads();
}

// per-CTA shared scratch of the eigen-solves
struct DisShared {
  double red[256];
  double rc[128];
  double2 rse[128];
  int rp[128], rq[128];
  int ord[128];
  double ev[128];
  int sel[128];
  int flag;
  __device__ JacobiScratch js() { return JacobiScratch{red, rc, rse, rp, rq}; }
};

// ---- dis_project (:1173-1429) and internal_slim_m (:453-529).  The projections arrive
// in U[0] (the reference passes them in u_matrix_opt); U_opt replaces them.
__global__ void __launch_bounds__(256) k_dis_project(DisDev D) {
  __shared__ DisShared sh;
  const int k = blockIdx.x;
  const int nb = D.nb, W = D.W, n = D.ndim[k], f = D.nfirst[k], B = D.B;
  const size_t NN = (size_t)nb * nb;
  double2* ws = D.ws + (size_t)k * kWs * NN;
  double2* Ak = D.A + (size_t)k * nb * W;
  double2* Uk = D.U[0] + (size_t)k * nb * W;
  for (int e = threadIdx.x; e < nb * W; e += blockDim.x) {
    const int i = e % nb, j = e / nb;
    ws[e] = (i < n) ? Uk[(size_t)j * nb + f + i] : cmk(0, 0);
  }
  for (int b = 0; b < B; ++b) {
    const int k2 = D.nnlist[k * B + b];
    const int n2 = D.ndim[k2], f2 = D.nfirst[k2];
    const double2* Mr = D.Mraw + ((size_t)k * B + b) * NN;
    double2* Mw = D.Mw + ((size_t)k * B + b) * NN;
    for (int e = threadIdx.x; e < (int)NN; e += blockDim.x) {
      const int i = e % nb, j = e / nb;
      Mw[e] = (i < n && j < n2) ? Mr[(size_t)(f2 + j) * nb + f + i] : cmk(0, 0);
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nb * W; e += blockDim.x) Ak[e] = ws[e];
  __syncthreads();
  cta_polar(ws + 5 * NN, nb, Ak, nb, n, W, ws + NN, ws + 2 * NN, ws + 3 * NN, ws + 4 * NN, sh.js(), &sh.flag);
  for (int e = threadIdx.x; e < nb * W; e += blockDim.x) {
    const int i = e % nb;
    Uk[e] = (i < n) ? ws[5 * NN + e] : cmk(0, 0);
  }
  if (threadIdx.x == 0) D.status[k] = sh.flag;
}

// ---- dis_proj_froz (:1431-1891): keep the frozen states, complete them with the leading
// eigenvectors of Q P Q (P = U U^H of the projected subspace, Q onto the non-frozen
// states), with the reference's choice among zero eigenvalues.  In place on U[0].
__global__ void __launch_bounds__(256) k_dis_froz(DisDev D) {
  __shared__ DisShared sh;
  __shared__ int nsel;
  const int k = blockIdx.x;
  const int nb = D.nb, W = D.W, n = D.ndim[k], nf = D.nfroz[k], ff = D.ffirst[k];
  if (nf == 0) return;
  const size_t NN = (size_t)nb * nb;
  double2* ws = D.ws + (size_t)k * kWs * NN;
  double2* Uk = D.U[0] + (size_t)k * nb * W;
  double2 *H = ws, *V = ws + NN;
  if (W > nf) {
    cta_zgemm(H, n, Uk, nb, false, Uk, nb, true, n, n, W);   // P = U U^H
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const bool fi = (i >= ff && i < ff + nf), fj = (j >= ff && j < ff + nf);
      if (fi || fj) H[e] = cmk(0, 0);
    }
    __syncthreads();
    const int sw = cta_jacobi(H, V, n, 60, sh.red, sh.rc, sh.rse, sh.rp, sh.rq);
    sort_eigs(H, n, sh.ord, sh.ev);
    if (threadIdx.x == 0) {
      const int need = W - nf;
      const int il = n - need;   // 0-based first of the leading ones (ascending)
      int nzero = 0, goods = 0;
      for (int j = n - 1; j >= il; --j) {
        if (sh.ev[sh.ord[j]] < 1e-8) ++nzero;
        else ++goods;
      }
      int cnt = 0;
      if (nzero == 0) {
        for (int j = il; j < n; ++j) sh.sel[cnt++] = sh.ord[j];
      } else {
        for (int j = n - 1; j > n - 1 - goods; --j) sh.sel[cnt++] = sh.ord[j];
        for (int z = 0; z < nzero; ++z) {
          for (int jj = n - 1; jj >= 0; --jj) {
            const int v = sh.ord[jj];
            bool used = false;
            for (int c = 0; c < cnt; ++c) used = used || (sh.sel[c] == v);
            if (used) continue;
            bool take = true;
            for (int m = 0; m < nf && take; ++m) {
              double2 t = cmk(0, 0);
              for (int j = 0; j < n; ++j) cfmac(t, Uk[(size_t)m * nb + j], V[(size_t)v * n + j]);
              if (sqrt(cabs2(t)) > 1e-8) take = false;
            }
            if (take) {
              sh.sel[cnt++] = v;
              break;
            }
          }
        }
      }
      nsel = cnt;
      if (sw < 0) D.status[k] = 2;
      if (cnt < need) D.status[k] = 3;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nb * (W - nf); e += blockDim.x) {
      const int i = e % nb, c = e / nb;
      Uk[(size_t)(nf + c) * nb + i] = (i < n && c < nsel) ? V[(size_t)sh.sel[c] * n + i] : cmk(0, 0);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nb * nf; e += blockDim.x) {
    const int i = e % nb, l = e / nb;
    Uk[(size_t)l * nb + i] = cmk(i == ff + l ? 1.0 : 0.0, 0.0);
  }
}

// ---- internal_zmatrix (:2922-2988), kept on every window state: Zf(k) = sum_b w_b C_b C_b^H
// with C_b = M_w(k,b) U_opt(k+b) (n x W).  The reference's Z is the block of Zf on the
// non-frozen states; the rest gives the Omega_I parts without a second pass over the
// overlaps:  sum_b w_b |U(k)^H M_w U(k+b)|_F^2 = tr(U^H Zf U), and for a frozen column
// e_f of U the row sum is Zf_ff.  Upper triangle summed, lower mirrored.  With
// want_omega, also wk[k] = W wbtot - Re tr(U^H Zf U) (Omega_I(i) part, :2480-2500).
__global__ void __launch_bounds__(256) k_dis_z(DisDev D, int cur, int to_in, int want_omega) {
  __shared__ double red[256];
  const int k = blockIdx.x;
  const int nb = D.nb, W = D.W, n = D.ndim[k], B = D.B;
  const size_t NN = (size_t)nb * nb;
  double2* ws = D.ws + (size_t)k * kWs * NN;
  double2* Zacc = ws + NN;
  double2* Z = (to_in ? D.Zin : D.Zout) + (size_t)k * NN;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) Zacc[e] = cmk(0, 0);
  for (int b = 0; b < B; ++b) {
    const int k2 = D.nnlist[k * B + b];
    const int n2 = D.ndim[k2];
    const double2* Mw = D.Mw + ((size_t)k * B + b) * NN;
    const double2* U2 = D.U[cur] + (size_t)k2 * nb * W;
    __syncthreads();
    cta_zgemm(ws, nb, Mw, nb, false, U2, nb, false, n, W, n2);   // C_b (n x W)
    __syncthreads();
    const double w = D.wb[b];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int p = e % n, q = e / n;
      if (p > q) continue;
      double2 acc = cmk(0, 0);
      for (int l = 0; l < W; ++l) cfma(acc, ws[(size_t)l * nb + p], cconj(ws[(size_t)l * nb + q]));
      Zacc[e] = cadd(Zacc[e], cscale(acc, w));
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int p = e % n, q = e / n;
    Z[(size_t)q * nb + p] = (p <= q) ? Zacc[e] : cconj(Zacc[(size_t)p * n + q]);
  }
  if (!want_omega) return;
  __syncthreads();
  // tr(U^H Zf U) = sum_{j} sum_p conj(U_pj) (Zf U)_pj
  const double2* Uk = D.U[cur] + (size_t)k * nb * W;
  double t = 0.0;
  for (int e = threadIdx.x; e < n * W; e += blockDim.x) {
    const int p = e % n, j = e / n;
    double2 acc = cmk(0, 0);
    for (int q = 0; q < n; ++q) cfma(acc, Z[(size_t)q * nb + p], Uk[(size_t)j * nb + q]);
    const double2 u = Uk[(size_t)j * nb + p];
    t += u.x * acc.x + u.y * acc.y;
  }
  t = block_sum(t, red);
  if (threadIdx.x == 0) D.wk[k] = (double)W * D.wbtot - t;
}

// ---- one step of dis_extract (:2160-2470): mix Z on the non-frozen states, diagonalise,
// new U_opt into U[cur^1], and the Omega_I(i-1) part of this k:
//   W wbtot - sum_{frozen f} Zf_ff (old U) - sum of the selected eigenvalues.
// Dynamic shared memory: the m x m eigenproblem (H, V) of the largest m over k.
__global__ void __launch_bounds__(256) k_dis_step(DisDev D, int cur, int it) {
  __shared__ DisShared sh;
  extern __shared__ double2 dsm[];
  const int k = blockIdx.x;
  const int nb = D.nb, W = D.W, n = D.ndim[k], nf = D.nfroz[k], ff = D.ffirst[k];
  const size_t NN = (size_t)nb * nb;
  const double2* Uo = D.U[cur] + (size_t)k * nb * W;
  double2* Un = D.U[cur ^ 1] + (size_t)k * nb * W;
  double2* Zi = D.Zin + (size_t)k * NN;
  const double2* Zo = D.Zout + (size_t)k * NN;
  // Zf of the old U_opt: Zin before the first mixing, Zout afterwards
  const double2* Zold = (it > 1) ? Zo : Zi;
  double wk1 = (double)W * D.wbtot;
  if (threadIdx.x == 0)
    for (int l = 0; l < nf; ++l) wk1 -= Zold[(size_t)(ff + l) * nb + ff + l].x;
  // frozen columns carry over; the others are rebuilt below
  for (int e = threadIdx.x; e < nb * W; e += blockDim.x) {
    const int c = e / nb;
    Un[e] = (c < nf || W <= nf) ? Uo[e] : cmk(0, 0);
  }
  if (W > nf) {
    const int m = n - nf;
    const int* nfi = D.nfidx + (size_t)k * nb;
    if (it > 1) {
      for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int p = e % m, q = e / m;
        if (p <= q) {
          const size_t o = (size_t)nfi[q] * nb + nfi[p];
          Zi[o] = cadd(cscale(Zo[o], D.mix), cscale(Zi[o], 1.0 - D.mix));
        }
      }
      __syncthreads();
    }
    const size_t mm = (size_t)m * m;
    double2 *H = dsm, *V = dsm + mm, *T = dsm + 2 * mm;
    double2* Vz = D.Vz + (size_t)k * NN;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int p = e % m, q = e / m;
      H[e] = (p <= q) ? Zi[(size_t)nfi[q] * nb + nfi[p]] : cconj(Zi[(size_t)nfi[p] * nb + nfi[q]]);
    }
    __syncthreads();
    // Z moves little from one iteration to the next: rotate it into the previous
    // eigenbasis, H = Vz^H Z Vz (Hermitised), so Jacobi starts near-diagonal
    const bool warm = it > 1;
    if (warm) {
      cta_zgemm(T, m, H, m, false, Vz, m, false, m, m, m);
      __syncthreads();
      cta_zgemm(H, m, Vz, m, true, T, m, false, m, m, m);
      __syncthreads();
      for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int p = e % m, q = e / m;
        if (p < q) {
          const double2 a = H[(size_t)q * m + p], b = cconj(H[(size_t)p * m + q]);
          const double2 h = cscale(cadd(a, b), 0.5);
          H[(size_t)q * m + p] = h;
          H[(size_t)p * m + q] = cconj(h);
        } else if (p == q) {
          H[e].y = 0.0;
        }
      }
      __syncthreads();
    }
    const int sw = cta_jacobi(H, V, m, 60, sh.red, sh.rc, sh.rse, sh.rp, sh.rq, 1.0e-30);
    sort_eigs(H, m, sh.ord, sh.ev);
    if (warm) {
      cta_zgemm(T, m, Vz, m, false, V, m, false, m, m, m);   // eigenvectors of Z
      __syncthreads();
    } else {
      T = V;
    }
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) Vz[e] = T[e];
    const int j0 = n - W, j1 = n - nf;   // selected ascending positions [j0, j1)
    if (threadIdx.x == 0) {
      for (int j = j0; j < j1; ++j) wk1 -= sh.ev[sh.ord[j]];
      if (sw < 0) D.status[k] = 2;
      atomicMax(D.max_sweeps, sw);
    }
    for (int e = threadIdx.x; e < m * (j1 - j0); e += blockDim.x) {
      const int i = e % m, c = e / m;
      Un[(size_t)(nf + c) * nb + nfi[i]] = T[(size_t)sh.ord[j0 + c] * m + i];
    }
  }
  if (threadIdx.x == 0) D.wk1[k] = wk1;
}

// ---- subspace Hamiltonian gauge (:2560-2640): U_opt <- U_opt V with V the eigenvectors
// (ascending) of U_opt^H diag(eig) U_opt
__global__ void __launch_bounds__(256) k_dis_gauge(DisDev D, int cur) {
  __shared__ DisShared sh;
  const int k = blockIdx.x;
  const int nb = D.nb, W = D.W, n = D.ndim[k];
  const size_t NN = (size_t)nb * nb;
  double2* ws = D.ws + (size_t)k * kWs * NN;
  double2* Uk = D.U[cur] + (size_t)k * nb * W;
  const double* e = D.eig + (size_t)k * nb;
  double2 *EU = ws, *H = ws + NN, *V = ws + 2 * NN, *R = ws + 3 * NN;
  for (int x = threadIdx.x; x < n * W; x += blockDim.x) {
    const int i = x % n, j = x / n;
    EU[(size_t)j * nb + i] = cscale(Uk[(size_t)j * nb + i], e[i]);
  }
  __syncthreads();
  cta_zgemm(H, W, Uk, nb, true, EU, nb, false, W, W, n);
  __syncthreads();
  const int sw = cta_jacobi(H, V, W, 60, sh.red, sh.rc, sh.rse, sh.rp, sh.rq);
  sort_eigs(H, W, sh.ord, sh.ev);
  for (int x = threadIdx.x; x < n * W; x += blockDim.x) {
    const int i = x % n, j = x / n;
    double2 acc = cmk(0, 0);
    for (int l = 0; l < W; ++l) cfma(acc, Uk[(size_t)l * nb + i], V[(size_t)sh.ord[j] * W + l]);
    R[(size_t)j * nb + i] = acc;
  }
  __syncthreads();
  for (int x = threadIdx.x; x < n * W; x += blockDim.x) {
    const int i = x % n, j = x / n;
    Uk[(size_t)j * nb + i] = R[(size_t)j * nb + i];
  }
  if (threadIdx.x == 0 && sw < 0) D.status[k] = 2;
}

// ---- internal_find_u (:531-698): U0 = polar factor of U_opt^H A
__global__ void __launch_bounds__(256) k_dis_findu(DisDev D, int cur) {
  __shared__ DisShared sh;
  const int k = blockIdx.x;
  const int nb = D.nb, W = D.W, n = D.ndim[k];
  const size_t NN = (size_t)nb * nb;
  double2* ws = D.ws + (size_t)k * kWs * NN;
  const double2* Uk = D.U[cur] + (size_t)k * nb * W;
  const double2* Ak = D.A + (size_t)k * nb * W;
  cta_zgemm(ws, W, Uk, nb, true, Ak, nb, false, W, W, n);
  __syncthreads();
  cta_polar(D.U0 + (size_t)k * W * W, W, ws, W, W, W, ws + NN, ws + 2 * NN, ws + 3 * NN, ws + 4 * NN, sh.js(), &sh.flag);
  if (threadIdx.x == 0 && sh.flag) D.status[k] = 10 + sh.flag;
}

// ---- dis_main's M_opt = U_opt^H M U_opt' (:220-235) and setup_m_loc's U0^H M_opt U0', per (k,b)
__global__ void __launch_bounds__(256) k_dis_rotate(DisDev D, int cur) {
  const int kb = blockIdx.x;
  const int k = kb / D.B;
  const int nb = D.nb, W = D.W, n = D.ndim[k];
  const int k2 = D.nnlist[kb];
  const int n2 = D.ndim[k2];
  const size_t NN = (size_t)nb * nb;
  extern __shared__ double2 sm[];   // W x nb + 2 W x W
  double2 *T1 = sm, *T2 = sm + (size_t)W * nb, *T3 = T2 + (size_t)W * W;
  const double2* Mw = D.Mw + (size_t)kb * NN;
  const double2* Uk = D.U[cur] + (size_t)k * nb * W;
  const double2* U2 = D.U[cur] + (size_t)k2 * nb * W;
  cta_zgemm(T1, W, Uk, nb, true, Mw, nb, false, W, n2, n);      // W x n2
  __syncthreads();
  cta_zgemm(T2, W, T1, W, false, U2, nb, false, W, W, n2);      // M_opt (W x W)
  __syncthreads();
  cta_zgemm(T3, W, D.U0 + (size_t)k * W * W, W, true, T2, W, false, W, W, W);
  __syncthreads();
  cta_zgemm(D.M0 + (size_t)kb * W * W, W, T3, W, false, D.U0 + (size_t)k2 * W * W, W, false, W, W, W);
}

// ---- symmetry-adapted mode (src/sitesym.F90, src/disentangle.F90:151-157, :186-190,
// :2193-2298, :2404-2411, :2504-2513, :627-629, :688-692).  One CTA per irreducible k.

// symmetrize_ukirr (src/sitesym.F90:392-497) on U (n rows used, leading dimension ld, W
// columns) at irreducible ir: the little group's average of d^+ U D, made unitary by
// orthogonalize_u's polar factor, until sum |ngk I - sum U^+ d^+ U D| < sym_eps (100
// passes).  d: band-representation slots with leading dimension ldd (their top-left
// n x n is used).  ws: 8 scratch matrices of ld x W (ld >= W).  Returns 0, 1 (not
// converged) or 2 (polar factor failed).
__device__ int dis_sym_ukirr(const DisDev& D, int ir, double2* U, int ld, int n, const double2* dslots, int ldd,
                             double2* ws, DisShared& sh) {
  const int W = D.W;
  const size_t L = (size_t)ld * W, WW = (size_t)W * W, DD = (size_t)ldd * ldd;
  double2 *Us = ws, *A = ws + L, *Bm = ws + 2 * L, *C2 = ws + 3 * L, *S = ws + 4 * L, *V = ws + 5 * L,
          *T = ws + 6 * L, *Y = ws + 7 * L;
  const int g0 = D.sym_goff[ir], g1 = D.sym_goff[ir + 1];
  const int ngk = g1 - g0;
  __syncthreads();
  if (ngk == 1) {
    cta_polar(U, ld, U, ld, n, W, S, V, T, Y, sh.js(), &sh.flag);
    return sh.flag ? 2 : 0;
  }
  for (int it = 1; it <= 100; ++it) {
    for (int e = threadIdx.x; e < (int)L; e += blockDim.x) Us[e] = cmk(0, 0);
    for (int e = threadIdx.x; e < (int)WW; e += blockDim.x) C2[e] = cmk((e % W) == (e / W) ? (double)ngk : 0.0, 0.0);
    for (int g = g0; g < g1; ++g) {
      const int slot = D.sym_grp[2 * g + 1];
      const double2* Dm = D.sym_d + (size_t)slot * WW;
      const double2* dm = dslots + (size_t)slot * DD;
      __syncthreads();
      cta_zgemm(A, ld, U, ld, false, Dm, W, false, n, W, W);        // cmat_sub = U D
      __syncthreads();
      cta_zgemm(Bm, ld, dm, ldd, true, A, ld, false, n, W, n);      // cmat = d^+ cmat_sub
      __syncthreads();
      for (int e = threadIdx.x; e < n * W; e += blockDim.x) {
        const int i = e % n, j = e / n;
        Us[(size_t)j * ld + i] = cadd(Us[(size_t)j * ld + i], Bm[(size_t)j * ld + i]);
      }
      for (int e = threadIdx.x; e < (int)WW; e += blockDim.x) {
        const int i = e % W, j = e / W;
        double2 acc = cmk(0, 0);
        for (int l = 0; l < n; ++l) cfmac(acc, U[(size_t)i * ld + l], Bm[(size_t)j * ld + l]);   // (U^+ cmat)_ij
        C2[e] = csub(C2[e], acc);
      }
    }
    __syncthreads();
    double diff = 0.0;
    for (int e = threadIdx.x; e < (int)WW; e += blockDim.x) diff += sqrt(cabs2(C2[e]));
    diff = block_sum(diff, sh.red);
    if (diff < D.sym_eps) return 0;
    if (it == 100) return 1;
    const double inv = 1.0 / (double)ngk;
    for (int e = threadIdx.x; e < n * W; e += blockDim.x) {
      const int i = e % n, j = e / n;
      Us[(size_t)j * ld + i] = cscale(Us[(size_t)j * ld + i], inv);
    }
    __syncthreads();
    cta_polar(U, ld, Us, ld, n, W, S, V, T, Y, sh.js(), &sh.flag);
    if (sh.flag) return 2;
  }
  return 1;
}

// sitesym_symmetrize_u_matrix (src/sitesym.F90:104-192).  mode 0: U_opt in U[buf]
// (window rows n = ndim(k_ir), d = the band slots); mode 1: the initial U (W x W, d = D
// after sitesym_replace_d_matrix_band).  Then U(R k) = d U(k_ir) D^+ over the star.
__global__ void __launch_bounds__(256) k_dis_sym_u(DisDev D, int buf, int mode) {
  __shared__ DisShared sh;
  const int ir = blockIdx.x;
  const int nb = D.nb, W = D.W;
  const int ik = D.sym_ik[ir];
  const size_t NN = (size_t)nb * nb, WW = (size_t)W * W;
  double2* ws = D.sym_ws + (size_t)ir * kDisSymWs * NN;
  const int ld = mode ? W : nb;
  const int n = mode ? W : D.ndim[ik];
  const double2* dslots = mode ? D.sym_d : D.sym_db;
  const int ldd = mode ? W : nb;
  double2* base = mode ? D.U0 : D.U[buf];
  const size_t blk = mode ? WW : (size_t)nb * W;
  double2* U = base + (size_t)ik * blk;
  const int status = dis_sym_ukirr(D, ir, U, ld, n, dslots, ldd, ws, sh);
  __syncthreads();
  double2* A = ws + 8 * NN;
  for (int m = D.sym_moff[ir]; m < D.sym_moff[ir + 1]; ++m) {
    const int slot = D.sym_mem[2 * m + 1];
    const double2* Dm = D.sym_d + (size_t)slot * WW;
    const double2* dm = dslots + (size_t)slot * ldd * ldd;
    double2* Um = base + (size_t)D.sym_mem[2 * m] * blk;
    cta_zgemm(A, ld, dm, ldd, false, U, ld, false, n, W, n);        // d U
    __syncthreads();
    cta_zgemm(Um, ld, A, ld, false, Dm, W, true, n, W, W);          // ... D^+
    __syncthreads();
  }
  if (threadIdx.x == 0 && status) D.sym_status[ir] = status + 10 * mode;
}

// sitesym_symmetrize_zmatrix (src/sitesym.F90:331-391) on Zin (which = 0) or Zout: at each
// irreducible k, Z += d^+ Z(Rk) d over the star's first occurrences, then the little
// group's d^+ Z d of that sum, divided by the group's order (window block nd x nd).
__global__ void __launch_bounds__(256) k_dis_sym_z(DisDev D, int which) {
  const int ir = blockIdx.x;
  const int nb = D.nb;
  const int ik = D.sym_ik[ir];
  const int nd = D.ndim[ik];
  const size_t NN = (size_t)nb * nb;
  double2* Zb = which ? D.Zout : D.Zin;
  double2* Z = Zb + (size_t)ik * NN;
  double2* ws = D.sym_ws + (size_t)ir * kDisSymWs * NN;
  double2 *C1 = ws, *C2 = ws + NN, *Tmp = ws + 2 * NN;
  for (int m = D.sym_moff[ir]; m < D.sym_moff[ir + 1]; ++m) {
    const double2* dm = D.sym_db + (size_t)D.sym_mem[2 * m + 1] * NN;
    const double2* Zm = Zb + (size_t)D.sym_mem[2 * m] * NN;
    __syncthreads();
    cta_zgemm(C1, nb, Zm, nb, false, dm, nb, false, nd, nd, nd);    // cmat1 = Z(Rk) d
    __syncthreads();
    cta_zgemm(C2, nb, dm, nb, true, C1, nb, false, nd, nd, nd);     // cmat2 = d^+ cmat1
    __syncthreads();
    for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
      const size_t o = (size_t)(e / nd) * nb + e % nd;
      Z[o] = cadd(Z[o], C2[o]);
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
    const size_t o = (size_t)(e / nd) * nb + e % nd;
    Tmp[o] = Z[o];
  }
  const int g0 = D.sym_goff[ir], g1 = D.sym_goff[ir + 1];
  for (int g = g0; g < g1; ++g) {
    if (D.sym_grp[2 * g] == 0) continue;    // isym = 1 is not part of this sum
    const double2* dm = D.sym_db + (size_t)D.sym_grp[2 * g + 1] * NN;
    __syncthreads();
    cta_zgemm(C1, nb, Tmp, nb, false, dm, nb, false, nd, nd, nd);
    __syncthreads();
    cta_zgemm(C2, nb, dm, nb, true, C1, nb, false, nd, nd, nd);
    __syncthreads();
    for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
      const size_t o = (size_t)(e / nd) * nb + e % nd;
      Z[o] = cadd(Z[o], C2[o]);
    }
  }
  __syncthreads();
  const double inv = 1.0 / (double)(g1 - g0);
  for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
    const size_t o = (size_t)(e / nd) * nb + e % nd;
    Z[o] = cscale(Z[o], inv);
  }
}

// The eigenvector of the larger eigenvalue of H v = w S v (2 x 2 Hermitian, S positive
// definite, both packed as (11, 12, 22)), S-normalised, with a real non-negative second
// component -- the phase ZHPGVX returns (zhptrd's reflector leaves the last coordinate
// alone).  Through the Cholesky factor S = L L^+.
__device__ void gen_eig2_larger(double h11, double2 h12, double h22, double s11, double2 s12, double s22,
                                double2* v) {
  // S = L L^+, L = [l11 0; l21 l22];  L^{-1} = [1/l11 0; i10 1/l22]
  const double l11 = sqrt(s11);
  const double2 l21 = cscale(cconj(s12), 1.0 / l11);
  const double l22 = sqrt(fmax(s22 - cabs2(l21), 1e-300));
  const double2 i10 = cscale(l21, -1.0 / (l11 * l22));
  // C = L^{-1} H L^{-+}: first M1 = L^{-1} H, then C = M1 L^{-+}, L^{-+} = [1/l11 conj(i10); 0 1/l22]
  const double2 m10 = cadd(cscale(i10, h11), cscale(cconj(h12), 1.0 / l22));
  const double2 m11 = cadd(cmul(i10, h12), cmk(h22 / l22, 0.0));
  const double c00 = h11 / s11;
  const double2 c10 = cscale(m10, 1.0 / l11);
  const double c11 = cadd(cmul(m10, cconj(i10)), cscale(m11, 1.0 / l22)).x;
  // the larger eigenvalue of [c00 conj(c10); c10 c11] and its eigenvector
  const double hm = 0.5 * (c00 - c11);
  const double lam = 0.5 * (c00 + c11) + sqrt(hm * hm + cabs2(c10));
  double2 y0, y1;
  if (cabs2(c10) > 0.0) {
    y0 = cconj(c10);                 // (C - lam) y = 0 from the first row
    y1 = cmk(lam - c00, 0.0);
  } else {
    y0 = cmk(c00 >= c11 ? 1.0 : 0.0, 0.0);
    y1 = cmk(c00 >= c11 ? 0.0 : 1.0, 0.0);
  }
  const double ny = sqrt(cabs2(y0) + cabs2(y1));
  y0 = cscale(y0, 1.0 / ny);
  y1 = cscale(y1, 1.0 / ny);
  // v = L^{-+} y
  const double2 v0 = cadd(cscale(y0, 1.0 / l11), cmul(cconj(i10), y1));
  const double2 v1 = cscale(y1, 1.0 / l22);
  // phase: second component real, >= 0
  const double a = sqrt(cabs2(v1));
  if (a > 0.0) {
    const double2 ph = cscale(cconj(v1), 1.0 / a);
    v[0] = cmul(v0, ph);
    v[1] = cmk(a, 0.0);
  } else {
    v[0] = v0;
    v[1] = v1;
  }
}

// dis_extract's refinement at an irreducible k (:2289-2298, sitesym_dis_extract_symmetry
// src/sitesym.F90:550-695): Z mixing (:2209-2228), then up to 50 passes of ZU = Z U,
// lambda = U^+ Z U, dU = ZU - U lambda (done when sum |dU| < 1e-10), each column moved to
// the larger solution of the 2 x 2 problem in span(u_i, dU_i), symmetrize_ukirr.
// Omega_I(i-1) part: W wbtot nsym / ngk - Re tr lambda.  The star's reducible k keep
// their U_opt (symmetrised afterwards) and add nothing.
__global__ void __launch_bounds__(256) k_dis_sym_step(DisDev D, int cur, int it) {
  __shared__ DisShared sh;
  __shared__ double s_h[8];
  __shared__ double2 s_v[2];
  __shared__ double s_red8[8][256];
  const int ir = blockIdx.x;
  const int nb = D.nb, W = D.W;
  const int k = D.sym_ik[ir];
  const int n = D.ndim[k];
  const size_t NN = (size_t)nb * nb, L = (size_t)nb * W;
  double2* Zi = D.Zin + (size_t)k * NN;
  const double2* Zo = D.Zout + (size_t)k * NN;
  double2* ws = D.sym_ws + (size_t)ir * kDisSymWs * NN;
  double2 *U = ws, *ZU = ws + NN, *dU = ws + 2 * NN, *lam = ws + 3 * NN, *Un = ws + 4 * NN, *Zh = ws + 5 * NN,
          *Zd = ws + 6 * NN;
  double2* uws = ws + 7 * NN;   // 8 blocks for dis_sym_ukirr
  // the star's reducible k: U_opt carried over, no Omega_I(i-1) part
  for (int m = D.sym_moff[ir]; m < D.sym_moff[ir + 1]; ++m) {
    const int km = D.sym_mem[2 * m];
    const double2* src = D.U[cur] + (size_t)km * L;
    double2* dst = D.U[cur ^ 1] + (size_t)km * L;
    for (int e = threadIdx.x; e < (int)L; e += blockDim.x) dst[e] = src[e];
    if (threadIdx.x == 0) D.wk1[km] = 0.0;
  }
  if (it > 1) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int p = e % n, q = e / n;
      if (p <= q) {
        const size_t o = (size_t)q * nb + p;
        Zi[o] = cadd(cscale(Zo[o], D.mix), cscale(Zi[o], 1.0 - D.mix));
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int p = e % n, q = e / n;
    Zh[(size_t)q * nb + p] = (p <= q) ? Zi[(size_t)q * nb + p] : cconj(Zi[(size_t)p * nb + q]);
  }
  const double2* Uo = D.U[cur] + (size_t)k * L;
  for (int e = threadIdx.x; e < (int)L; e += blockDim.x) U[e] = Uo[e];
  int status = 0;
  for (int pass = 0; pass < 50; ++pass) {
    __syncthreads();
    cta_zgemm(ZU, nb, Zh, nb, false, U, nb, false, n, W, n);        // Z U
    __syncthreads();
    cta_zgemm(lam, W, U, nb, true, ZU, nb, false, W, W, n);         // lambda = U^+ Z U
    __syncthreads();
    cta_zgemm(dU, nb, U, nb, false, lam, W, false, n, W, W);        // U lambda
    __syncthreads();
    double sa = 0.0;
    for (int e = threadIdx.x; e < n * W; e += blockDim.x) {
      const size_t o = (size_t)(e / n) * nb + e % n;
      dU[o] = csub(ZU[o], dU[o]);
      sa += sqrt(cabs2(dU[o]));
    }
    sa = block_sum(sa, sh.red);
    if (sa < 1e-10) break;
    for (int i = 0; i < W; ++i) {
      const double2 *u = U + (size_t)i * nb, *zu = ZU + (size_t)i * nb, *du = dU + (size_t)i * nb;
      for (int p = threadIdx.x; p < n; p += blockDim.x) {
        double2 acc = cmk(0, 0);
        for (int q = 0; q < n; ++q) cfma(acc, Zh[(size_t)q * nb + p], du[q]);
        Zd[p] = acc;
      }
      __syncthreads();
      // h11 = Re u^+ zu, h12 = zu^+ du, h22 = Re du^+ Z du, s11 = u^+ u, s12 = u^+ du, s22 = du^+ du
      double t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int p = threadIdx.x; p < n; p += blockDim.x) {
        t[0] += u[p].x * zu[p].x + u[p].y * zu[p].y;
        t[1] += zu[p].x * du[p].x + zu[p].y * du[p].y;
        t[2] += zu[p].x * du[p].y - zu[p].y * du[p].x;
        t[3] += du[p].x * Zd[p].x + du[p].y * Zd[p].y;
        t[4] += cabs2(u[p]);
        t[5] += u[p].x * du[p].x + u[p].y * du[p].y;
        t[6] += u[p].x * du[p].y - u[p].y * du[p].x;
        t[7] += cabs2(du[p]);
      }
      // the eight sums in one tree (blockDim is a power of two <= 256)
      for (int c = 0; c < 8; ++c) s_red8[c][threadIdx.x] = t[c];
      __syncthreads();
      for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
          for (int c = 0; c < 8; ++c) s_red8[c][threadIdx.x] += s_red8[c][threadIdx.x + h];
        __syncthreads();
      }
      if (threadIdx.x < 8) s_h[threadIdx.x] = s_red8[threadIdx.x][0];
      __syncthreads();
      const bool keep = fabs(s_h[7]) < 1e-10;
      if (threadIdx.x == 0 && !keep)
        gen_eig2_larger(s_h[0], cmk(s_h[1], s_h[2]), s_h[3], s_h[4], cmk(s_h[5], s_h[6]), s_h[7], s_v);
      __syncthreads();
      double2* un = Un + (size_t)i * nb;
      for (int p = threadIdx.x; p < nb; p += blockDim.x) {
        if (keep) un[p] = u[p];
        else un[p] = (p < n) ? cadd(cmul(s_v[0], u[p]), cmul(s_v[1], du[p])) : cmk(0, 0);
      }
      __syncthreads();
    }
    status = dis_sym_ukirr(D, ir, Un, nb, n, D.sym_db, nb, uws, sh);
    __syncthreads();
    for (int e = threadIdx.x; e < (int)L; e += blockDim.x) U[e] = Un[e];
    if (status) break;
  }
  __syncthreads();
  double2* Un_out = D.U[cur ^ 1] + (size_t)k * L;
  for (int e = threadIdx.x; e < (int)L; e += blockDim.x) Un_out[e] = U[e];
  double tr = 0.0;
  for (int j = threadIdx.x; j < W; j += blockDim.x) tr += lam[(size_t)j * W + j].x;
  tr = block_sum(tr, sh.red);
  if (threadIdx.x == 0) {
    const int ngk = D.sym_goff[ir + 1] - D.sym_goff[ir];
    D.wk1[k] = (double)W * D.wbtot * D.sym_nsym / ngk - tr;
    if (status) D.sym_status[ir] = status;
  }
}

}  // namespace

const char* dis_kernel_name(int i) {
  static const char* names[kDisKernels] = {"k_dis_project", "k_dis_froz", "k_dis_z", "k_dis_step",
                                           "k_dis_gauge", "k_dis_findu", "k_dis_rotate", "k_dis_sym"};
  return (i >= 0 && i < kDisKernels) ? names[i] : "";
}

#define DIS_CHECK(call)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
      rc = (e_ == cudaErrorMemoryAllocation) ? 2 : 1;                       \
      goto done;                                                            \
    }                                                                       \
  } while (0)

// dis_windows (src/disentangle.F90:851-1171) on the host: outer window [nfirst, +ndim),
// frozen states [ffirst, +nfroz) inside it, the non-frozen window states, and the
// window eigenvalues.  Returns 0 or 1 (fatal) with err set.
static int dis_windows(const DisControl& c, const double* eig, int nb, int W, int K, std::vector<int>& ndim,
                       std::vector<int>& nfirst, std::vector<int>& nfroz, std::vector<int>& ffirst,
                       std::vector<int>& nfidx, std::vector<double>& eigw, std::string& err) {
  ndim.assign(K, 0);
  nfirst.assign(K, 0);
  nfroz.assign(K, 0);
  ffirst.assign(K, 0);
  nfidx.assign((size_t)K * nb, 0);
  eigw.assign((size_t)K * nb, 0.0);
  for (int k = 0; k < K; ++k) {
    const double* e = eig + (size_t)k * nb;
    if (e[0] > c.win_max || e[nb - 1] < c.win_min) {
      err = "dis_windows: The outer energy window contains no eigenvalues";
      return 1;
    }
    int imin = -1, imax = -1;
    for (int i = 0; i < nb; ++i) {
      if (imin < 0) {
        if (e[i] >= c.win_min && e[i] <= c.win_max) imin = i;
        imax = i;
      }
      if (e[i] <= c.win_max) imax = i;
    }
    if (imin < 0) {
      err = "dis_windows: The outer energy window contains no eigenvalues";
      return 1;
    }
    ndim[k] = imax - imin + 1;
    nfirst[k] = imin;
    if (ndim[k] < W) {
      err = "dis_windows: Energy window contains fewer states than number of target WFs";
      return 1;
    }
    int fmin = -1, fmax = -2;
    if (c.frozen_states) {
      for (int i = imin; i <= imax; ++i) {
        if (fmin < 0) {
          if (e[i] >= c.froz_min && e[i] <= c.froz_max) fmin = fmax = i - imin;
        } else if (e[i] <= c.froz_max) {
          ++fmax;
        }
      }
    }
    nfroz[k] = (fmin >= 0) ? fmax - fmin + 1 : 0;
    ffirst[k] = (fmin >= 0) ? fmin : 0;
    if (nfroz[k] > W) {
      err = "dis_windows: More states in the frozen window than target WFs";
      return 1;
    }
    int cnt = 0;
    for (int j = 0; j < ndim[k]; ++j)
      if (!(nfroz[k] > 0 && j >= ffirst[k] && j < ffirst[k] + nfroz[k])) nfidx[(size_t)k * nb + cnt++] = j;
    for (int i = 0; i < ndim[k]; ++i) eigw[(size_t)k * nb + i] = e[imin + i];
  }
  return 0;
}

int dis_run(const DisSpec& s, DisResult& r, std::string& err) {
  const int nb = s.nb, W = s.W, K = s.K, B = s.B;
  if (nb < W || nb > 64 || W < 1 || K < 1 || B < 1) {
    err = "disentangle: the GPU engine needs num_wann <= num_bands <= 64";
    return 5;
  }
  const DisControl& c = s.ctl;
  if (c.conv_window < 0 || c.num_iter < 0) {
    err = "disentangle: dis_num_iter and dis_conv_window must be positive";
    return 5;
  }
  const cudaMemcpyKind in_kind = s.device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out_kind = s.device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  std::vector<int> ndim, nfirst, nfroz, ffirst, nfidx;
  std::vector<double> eigw, eig_host;
  const double* eig = s.eig;
  if (s.device) {
    // the windows are set up on the host: bring the band energies over first
    eig_host.resize((size_t)K * nb);
    cudaError_t e = cudaMemcpy(eig_host.data(), s.eig, eig_host.size() * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      err = std::string("disentangle: eigval copy: ") + cudaGetErrorString(e);
      return 1;
    }
    eig = eig_host.data();
  }
  {
    const int wrc = dis_windows(c, eig, nb, W, K, ndim, nfirst, nfroz, ffirst, nfidx, eigw, err);
    if (wrc) return wrc;
  }
  bool any_froz = false;
  for (int v : nfroz) any_froz = any_froz || v > 0;
  const int nir = s.sym_nir;
  if (nir > 0) {
    if (any_froz) {
      // dis_main (src/disentangle.F90:154-157)
      err = "in symmetry-adapted mode, frozen window not implemented yet";
      return 1;
    }
    const size_t nslot = s.sym_d.size() / (2 * (size_t)W * W);
    if (s.sym_ik.size() != (size_t)nir || s.sym_moff.size() != (size_t)nir + 1 ||
        s.sym_goff.size() != (size_t)nir + 1 || s.sym_mem.size() != 2 * (size_t)s.sym_moff[nir] ||
        s.sym_grp.size() != 2 * (size_t)s.sym_goff[nir] || nslot == 0 ||
        s.sym_db.size() != nslot * 2 * (size_t)nb * nb || s.sym_nsym < 1) {
      err = "disentangle: site symmetry tables missing or inconsistent";
      return 5;
    }
  }

  const auto t0 = std::chrono::steady_clock::now();
  int rc = 0;
  DisDev D{};
  void* arena = nullptr;
  std::vector<double> wk1(K), wk(K), history(c.conv_window, 0.0);
  std::vector<int> status(K);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t NN = (size_t)nb * nb;
  const size_t o_nn = take((size_t)K * B * 4), o_wb = take(B * 8), o_ndim = take(K * 4), o_nfirst = take(K * 4),
               o_nfroz = take(K * 4), o_ffirst = take(K * 4), o_nfidx = take((size_t)K * nb * 4),
               o_eig = take((size_t)K * nb * 8), o_mraw = take((size_t)K * B * NN * 16),
               o_mw = take((size_t)K * B * NN * 16), o_a = take((size_t)K * nb * W * 16),
               o_u0b = take((size_t)K * nb * W * 16), o_u1b = take((size_t)K * nb * W * 16),
               o_zin = take((size_t)K * NN * 16), o_zout = take((size_t)K * NN * 16),
               o_uw = take((size_t)K * W * W * 16), o_m0 = take((size_t)K * B * W * W * 16),
               o_ws = take((size_t)K * kWs * NN * 16), o_wk1 = take(K * 8), o_wk = take(K * 8),
               o_st = take(K * 4), o_vz = take((size_t)K * NN * 16), o_sw = take(4);
  // symmetry tables: ik, moff, mem, goff, grp, status; slot matrices; workspace
  std::vector<int> sym_ints;
  if (nir > 0) {
    for (auto* v : {&s.sym_ik, &s.sym_moff, &s.sym_mem, &s.sym_goff, &s.sym_grp})
      sym_ints.insert(sym_ints.end(), v->begin(), v->end());
    sym_ints.insert(sym_ints.end(), (size_t)nir, 0);
  }
  const size_t o_syi = take(sym_ints.size() * 4), o_syd = take(s.sym_d.size() * 8),
               o_sydb = take(s.sym_db.size() * 8), o_syws = take((size_t)nir * kDisSymWs * NN * 16);
  const size_t rot_smem = ((size_t)W * nb + 2 * (size_t)W * W) * 16;
  int mmax = 0;
  for (int k = 0; k < K; ++k) mmax = std::max(mmax, ndim[k] - nfroz[k]);
  const size_t step_smem = 3 * (size_t)mmax * mmax * 16;
  int cur = 0, it = 0;
  double womegai = 0.0;
  cudaStream_t st = s.stream;
  bool own_stream = false;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // launch with optional per-kernel event timing
  auto launch = [&](int id, auto&& fn) -> cudaError_t {
    if (s.prof_ms) cudaEventRecord(ev[0], st);
    fn();
    ++r.launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !s.prof_ms) return e;
    cudaEventRecord(ev[1], st);
    e = cudaEventSynchronize(ev[1]);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    s.prof_ms[id] += ms;
    if (s.prof_counts) ++s.prof_counts[id];
    return e;
  };
  r.launches = 0;
  if (!st) {
    DIS_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    own_stream = true;
  }
  if (s.prof_ms) {
    DIS_CHECK(cudaEventCreate(&ev[0]));
    DIS_CHECK(cudaEventCreate(&ev[1]));
  }
  // the attributes are process-wide: always the largest any call needs (nb <= 64), so
  // concurrent calls of different sizes never lower them under one another
  DIS_CHECK(cudaFuncSetAttribute(k_dis_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDisMaxSmem));
  DIS_CHECK(cudaFuncSetAttribute(k_dis_rotate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDisMaxSmem));
  DIS_CHECK(cudaMallocAsync(&arena, off, st));
  {
    char* a = (char*)arena;
    D.nb = nb;
    D.W = W;
    D.K = K;
    D.B = B;
    D.wbtot = s.wbtot;
    D.mix = c.mix_ratio;
    D.nnlist = (const int*)(a + o_nn);
    D.wb = (const double*)(a + o_wb);
    D.ndim = (const int*)(a + o_ndim);
    D.nfirst = (const int*)(a + o_nfirst);
    D.nfroz = (const int*)(a + o_nfroz);
    D.ffirst = (const int*)(a + o_ffirst);
    D.nfidx = (const int*)(a + o_nfidx);
    D.eig = (const double*)(a + o_eig);
    D.Mraw = (const double2*)(a + o_mraw);
    D.Mw = (double2*)(a + o_mw);
    D.A = (double2*)(a + o_a);
    D.U[0] = (double2*)(a + o_u0b);
    D.U[1] = (double2*)(a + o_u1b);
    D.Zin = (double2*)(a + o_zin);
    D.Zout = (double2*)(a + o_zout);
    D.U0 = (double2*)(a + o_uw);
    D.M0 = (double2*)(a + o_m0);
    D.ws = (double2*)(a + o_ws);
    D.wk1 = (double*)(a + o_wk1);
    D.wk = (double*)(a + o_wk);
    D.status = (int*)(a + o_st);
    D.Vz = (double2*)(a + o_vz);
    D.max_sweeps = (int*)(a + o_sw);
    D.sym_nir = nir;
    D.sym_nsym = s.sym_nsym;
    D.sym_eps = s.sym_eps;
    if (nir > 0) {
      int* si = (int*)(a + o_syi);
      size_t o = 0;
      D.sym_ik = si;
      D.sym_moff = si + (o += s.sym_ik.size());
      D.sym_mem = si + (o += s.sym_moff.size());
      D.sym_goff = si + (o += s.sym_mem.size());
      D.sym_grp = si + (o += s.sym_goff.size());
      D.sym_status = si + (o += s.sym_grp.size());
      D.sym_d = (const double2*)(a + o_syd);
      D.sym_db = (const double2*)(a + o_sydb);
      D.sym_ws = (double2*)(a + o_syws);
    }
  }
  if (nir > 0) {
    DIS_CHECK(cudaMemcpyAsync((void*)D.sym_ik, sym_ints.data(), sym_ints.size() * 4, cudaMemcpyHostToDevice, st));
    DIS_CHECK(cudaMemcpyAsync((void*)D.sym_d, s.sym_d.data(), s.sym_d.size() * 8, cudaMemcpyHostToDevice, st));
    DIS_CHECK(cudaMemcpyAsync((void*)D.sym_db, s.sym_db.data(), s.sym_db.size() * 8, cudaMemcpyHostToDevice, st));
  }
  DIS_CHECK(cudaMemcpyAsync((void*)D.nnlist, s.nnlist.data(), (size_t)K * B * 4, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.wb, s.wb.data(), B * 8, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.ndim, ndim.data(), K * 4, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.nfirst, nfirst.data(), K * 4, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.nfroz, nfroz.data(), K * 4, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.ffirst, ffirst.data(), K * 4, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.nfidx, nfidx.data(), (size_t)K * nb * 4, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.eig, eigw.data(), (size_t)K * nb * 8, cudaMemcpyHostToDevice, st));
  DIS_CHECK(cudaMemcpyAsync((void*)D.Mraw, s.M, (size_t)K * B * NN * 16, in_kind, st));
  DIS_CHECK(cudaMemcpyAsync(D.U[0], s.A, (size_t)K * nb * W * 16, in_kind, st));
  DIS_CHECK(cudaMemsetAsync(D.status, 0, K * 4, st));
  DIS_CHECK(cudaMemsetAsync(D.max_sweeps, 0, 4, st));
  DIS_CHECK(launch(kDisProject, [&] { k_dis_project<<<K, 256, 0, st>>>(D); }));
  if (any_froz) DIS_CHECK(launch(kDisFroz, [&] { k_dis_froz<<<K, 256, 0, st>>>(D); }));
  DIS_CHECK(cudaMemcpyAsync(status.data(), D.status, K * 4, cudaMemcpyDeviceToHost, st));
  DIS_CHECK(cudaStreamSynchronize(st));
  for (int k = 0; k < K; ++k) {
    if (status[k]) {
      err = status[k] == 3 ? "dis_proj_froz: Ortho-fix failed to find enough vectors"
                           : "dis_project: projections rank deficient or eigensolver failure at k-point " +
                                 std::to_string(k + 1);
      rc = 1;
      goto done;
    }
  }
  // symmetry-adapted U_opt (src/disentangle.F90:186-190)
  if (nir > 0) DIS_CHECK(launch(kDisSym, [&] { k_dis_sym_u<<<nir, 256, 0, st>>>(D, cur, 0); }));
  // ---- dis_extract iterations
  DIS_CHECK(launch(kDisZ, [&] { k_dis_z<<<K, 256, 0, st>>>(D, cur, 1, 0); }));
  if (nir > 0) DIS_CHECK(launch(kDisSym, [&] { k_dis_sym_z<<<nir, 256, 0, st>>>(D, 0); }));
  r.log.clear();
  r.converged = 0;
  for (it = 1; it <= c.num_iter; ++it) {
    if (nir > 0) {
      DIS_CHECK(launch(kDisSym, [&] { k_dis_sym_step<<<nir, 256, 0, st>>>(D, cur, it); }));
      DIS_CHECK(launch(kDisSym, [&] { k_dis_sym_u<<<nir, 256, 0, st>>>(D, cur ^ 1, 0); }));
    } else {
      DIS_CHECK(launch(kDisStep, [&] { k_dis_step<<<K, 256, step_smem, st>>>(D, cur, it); }));
    }
    DIS_CHECK(launch(kDisZ, [&] { k_dis_z<<<K, 256, 0, st>>>(D, cur ^ 1, 0, 1); }));
    if (nir > 0) DIS_CHECK(launch(kDisSym, [&] { k_dis_sym_z<<<nir, 256, 0, st>>>(D, 1); }));
    DIS_CHECK(cudaMemcpyAsync(wk1.data(), D.wk1, K * 8, cudaMemcpyDeviceToHost, st));
    DIS_CHECK(cudaMemcpyAsync(wk.data(), D.wk, K * 8, cudaMemcpyDeviceToHost, st));
    DIS_CHECK(cudaStreamSynchronize(st));
    cur ^= 1;
    double w1 = 0.0, w2 = 0.0;
    for (int k = 0; k < K; ++k) {
      w1 += wk1[k];
      w2 += wk[k];
    }
    w1 /= K;
    w2 /= K;
    womegai = w2;
    const double delta = w1 / w2 - 1.0;
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r.log.insert(r.log.end(), {(double)it, w1, w2, delta, secs});
    // internal_test_convergence (:2866-2920)
    if (c.conv_window == 0) {
    } else if (it <= c.conv_window) {
      history[it - 1] = delta;
    } else {
      for (int i = 0; i + 1 < c.conv_window; ++i) history[i] = history[i + 1];
      history[c.conv_window - 1] = delta;
    }
    if (it >= c.conv_window) {
      bool conv = true;
      for (double h : history) conv = conv && std::fabs(h) < c.conv_tol;
      if (conv) {
        r.converged = 1;
        break;
      }
    }
  }
  // the subspace-Hamiltonian gauge is kept out in the symmetry-adapted mode (:2675)
  if (nir == 0) DIS_CHECK(launch(kDisGauge, [&] { k_dis_gauge<<<K, 256, 0, st>>>(D, cur); }));
  DIS_CHECK(launch(kDisFindU, [&] { k_dis_findu<<<K, 256, 0, st>>>(D, cur); }));
  // symmetric initial U with d = D (sitesym_replace_d_matrix_band, :237, :688-692)
  if (nir > 0) DIS_CHECK(launch(kDisSym, [&] { k_dis_sym_u<<<nir, 256, 0, st>>>(D, cur, 1); }));
  DIS_CHECK(launch(kDisRotate, [&] { k_dis_rotate<<<K * B, 256, rot_smem, st>>>(D, cur); }));
  DIS_CHECK(cudaMemcpyAsync(status.data(), D.status, K * 4, cudaMemcpyDeviceToHost, st));
  DIS_CHECK(cudaMemcpyAsync(&r.max_sweeps, D.max_sweeps, 4, cudaMemcpyDeviceToHost, st));
  DIS_CHECK(cudaStreamSynchronize(st));
  for (int k = 0; k < K; ++k) {
    if (status[k]) {
      err = "disentangle: eigensolver failure or rank-deficient U_opt^H A at k-point " + std::to_string(k + 1);
      rc = 1;
      goto done;
    }
  }
  if (nir > 0) {
    std::vector<int> ss(nir);
    DIS_CHECK(cudaMemcpy(ss.data(), D.sym_status, nir * sizeof(int), cudaMemcpyDeviceToHost));
    for (int v : ss) {
      if (v % 10 == 1) {
        // set_error_unconv (src/sitesym.F90:478-486)
        err = "symmetrize_ukirr: not converged";
        rc = -1;
        goto done;
      }
      if (v) {
        err = " ERROR: IN ZGESVD IN orthogonalize_u";
        rc = 1;
        goto done;
      }
    }
  }
  if (s.uopt_out) DIS_CHECK(cudaMemcpyAsync(s.uopt_out, D.U[cur], (size_t)K * nb * W * 16, out_kind, st));
  if (s.u_out) DIS_CHECK(cudaMemcpyAsync(s.u_out, D.U0, (size_t)K * W * W * 16, out_kind, st));
  if (s.m_out) DIS_CHECK(copy_wblocks(s.m_out, nb, D.M0, W, W, K * B, out_kind, st));
  DIS_CHECK(cudaStreamSynchronize(st));
  r.omega_invariant = womegai;
  r.ndimwin = ndim;
  r.nfirstwin = nfirst;
done:
  if (arena) {
    cudaFreeAsync(arena, st);
    cudaStreamSynchronize(st);
  }
  if (ev[0]) cudaEventDestroy(ev[0]);
  if (ev[1]) cudaEventDestroy(ev[1]);
  if (own_stream) cudaStreamDestroy(st);
  return rc;
}

}  // namespace w90g
