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
};

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

}  // namespace

const char* dis_kernel_name(int i) {
  static const char* names[kDisKernels] = {"k_dis_project", "k_dis_froz", "k_dis_z", "k_dis_step",
                                           "k_dis_gauge", "k_dis_findu", "k_dis_rotate"};
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
  // ---- dis_extract iterations
  DIS_CHECK(launch(kDisZ, [&] { k_dis_z<<<K, 256, 0, st>>>(D, cur, 1, 0); }));
  r.log.clear();
  r.converged = 0;
  for (it = 1; it <= c.num_iter; ++it) {
    DIS_CHECK(launch(kDisStep, [&] { k_dis_step<<<K, 256, step_smem, st>>>(D, cur, it); }));
    DIS_CHECK(launch(kDisZ, [&] { k_dis_z<<<K, 256, 0, st>>>(D, cur ^ 1, 0, 1); }));
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
  DIS_CHECK(launch(kDisGauge, [&] { k_dis_gauge<<<K, 256, 0, st>>>(D, cur); }));
  DIS_CHECK(launch(kDisFindU, [&] { k_dis_findu<<<K, 256, 0, st>>>(D, cur); }));
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
