// CTA-wide building blocks shared by the FP64 kernels: deterministic block reductions
// and a parallel-ordered Jacobi eigensolver for small Hermitian matrices.
#pragma once
#include "w90g.cuh"

namespace w90g {

__device__ __forceinline__ double block_sum(double v, double* red) {
  // deterministic tree reduction over blockDim.x (power of two, <= 1024)
  int t = threadIdx.x;
  red[t] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (t < s) red[t] += red[t + s];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, double* red) {
  int t = threadIdx.x;
  red[t] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (t < s) red[t] = fmax(red[t], red[t + s]);
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

// ----------------------------------------------------------------------------
// Parallel-ordered cyclic Jacobi eigensolver for a Hermitian W x W matrix H (generic
// pointer, overwritten by its near-diagonal form); V receives the eigenvectors
// (columns).  Rotation for pair (p,q):  J = [[c, s e^{i phi}], [-s e^{-i phi}, c]],
// phi = arg(H_pq), (c, s) the real Jacobi rotation of [[H_pp, |H_pq|], [|H_pq|, H_qq]].
// Convergence: sum_{p != q} |H_pq|^2 <= 1e-30 ||H||_F^2.  With skip_rel > 0, pairs with
// |H_pq|^2 <= skip_rel ||H||_F^2 are left alone and a sweep that rotates no pair also ends
// the solve (the threshold-Jacobi rule: reachable at any size, where the plain criterion
// can sit at the roundoff floor of large matrices).
// Returns the number of sweeps used (or -1 when not converged within max_sweeps).
// ----------------------------------------------------------------------------
__device__ __noinline__ static int cta_jacobi(double2* H, double2* V, int W, int max_sweeps, double* red,
                          double* rc, double2* rse, int* rp, int* rq, double skip_rel = 0.0) {
  const int WW = W * W;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    V[e] = cmk((e % W) == (e / W) ? 1.0 : 0.0, 0.0);
  }
  const int n = (W + 1) & ~1;     // even number of players (one dummy when W is odd)
  const int npair = n / 2;
  __syncthreads();
  for (int sweep = 0; sweep <= max_sweeps; ++sweep) {
    double off = 0.0, fro = 0.0;
    for (int e = threadIdx.x; e < WW; e += blockDim.x) {
      const double a = cabs2(H[e]);
      fro += a;
      if ((e % W) != (e / W)) off += a;
    }
    off = block_sum(off, red);
    fro = block_sum(fro, red);
    if (off <= 1.0e-30 * fro || off == 0.0) return sweep;
    if (sweep == max_sweeps) break;
    const double thr = skip_rel * fro;
    int rotated = 0;
    for (int r = 0; r < n - 1; ++r) {
      for (int t = threadIdx.x; t < npair; t += blockDim.x) {
        int p, q;
        if (t == 0) {
          p = r;
          q = n - 1;
        } else {
          p = (r + t) % (n - 1);
          q = (r - t + (n - 1)) % (n - 1);
        }
        if (p > q) {
          const int x = p;
          p = q;
          q = x;
        }
        double c = 1.0;
        double2 se = cmk(0, 0);
        if (q < W) {
          const double2 b = H[q * W + p];
          const double ab = sqrt(cabs2(b));
          if (ab > 1.0e-300 && (skip_rel == 0.0 || ab * ab > thr)) {
            ++rotated;
            const double a = H[p * W + p].x, d = H[q * W + q].x;
            const double th = (d - a) / (2.0 * ab);
            const double tt = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(1.0 + th * th));
            c = 1.0 / sqrt(1.0 + tt * tt);
            const double s = tt * c;
            se = cmk(s * b.x / ab, s * b.y / ab);
          }
        }
        rp[t] = p;
        rq[t] = q;
        rc[t] = c;
        rse[t] = se;
      }
      __syncthreads();
      // columns: H <- H J, V <- V J
      for (int e = threadIdx.x; e < W * npair; e += blockDim.x) {
        const int i = e % W, t = e / W;
        const int p = rp[t], q = rq[t];
        if (q >= W) continue;
        const double c = rc[t];
        const double2 se = rse[t];
        const double2 hp = H[p * W + i], hq = H[q * W + i];
        // (HJ)_ip = c H_ip - conj(se) H_iq ; (HJ)_iq = se H_ip + c H_iq
        H[p * W + i] = csub(cscale(hp, c), cmul(cconj(se), hq));
        H[q * W + i] = cadd(cmul(se, hp), cscale(hq, c));
        const double2 vp = V[p * W + i], vq = V[q * W + i];
        V[p * W + i] = csub(cscale(vp, c), cmul(cconj(se), vq));
        V[q * W + i] = cadd(cmul(se, vp), cscale(vq, c));
      }
      __syncthreads();
      // rows: H <- J^H H
      for (int e = threadIdx.x; e < W * npair; e += blockDim.x) {
        const int j = e % W, t = e / W;
        const int p = rp[t], q = rq[t];
        if (q >= W) continue;
        const double c = rc[t];
        const double2 se = rse[t];
        const double2 hp = H[j * W + p], hq = H[j * W + q];
        // (J^H H)_pj = c H_pj - se H_qj ; (J^H H)_qj = conj(se) H_pj + c H_qj
        H[j * W + p] = csub(cscale(hp, c), cmul(se, hq));
        H[j * W + q] = cadd(cmul(cconj(se), hp), cscale(hq, c));
      }
      __syncthreads();
    }
    if (skip_rel > 0.0 && block_sum((double)rotated, red) == 0.0) return sweep + 1;
  }
  return -1;
}

}  // namespace w90g
