// Symmetry-adapted mode of wann_main (site_symmetry = T, src/sitesym.F90), isolated bands.
//
// The reference keeps the unknowns at the irreducible k-points and maps them onto each
// star with the representation matrices D(R, k_ir) of the Wannier functions (and d(R, k_ir)
// of the bands, for the initial U):
//   k_sym_grad  after k_grad: sitesym_symmetrize_gradient modes 1 and 2 (:195-278) -- the
//               star's gradients gathered onto k_ir, averaged over its little group, zero at
//               the reducible k -- and the CG partial sums of the symmetrised gradient;
//   k_sym_dir   after k_ctrl_search: the search direction D = coefG G + coefD D_prev formed
//               at k_ir and rotated onto the star, D(R k) = D(R,k) D(k) D(R,k)^+.  The exp
//               kernels then exponentiate every k: exp(s D X D^+) = D exp(s X) D^+, the
//               rotation sitesym_symmetrize_rotation (:281-328) applies to dU, so the M
//               update and U dU run unchanged;
//   k_sym_u     in the projection, after the Loewdin step: sitesym_symmetrize_u_matrix
//               (:104-192) -- symmetrize_ukirr's fixed-point iteration at k_ir (:392-497)
//               with the polar factor of orthogonalize_u (:500-548), then
//               U(R k) = d(R,k) U(k) D(R,k)^+ over the star.
// One CTA (256 threads) per (problem, irreducible k); the W x W work matrices live in a
// per-irreducible-k workspace in HBM (kSymWork matrices each; they stay in L2).  Tables are built on the host with
// the reference's first-occurrence order (capi.cpp): star members (k, slot) and the little
// group (isym, slot), slot indexing the stored D / d matrices.
#include "w90g.cuh"
#include "cta.cuh"

namespace w90g {

namespace {

// C = op(A) op(B), W x W column-major; op 'N' or conjugate transpose ('C')
template <bool CA, bool CB>
__device__ void sym_mm(double2* __restrict__ C, const double2* __restrict__ A, const double2* __restrict__ B, int W) {
  const int WW = W * W;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    const int i = e % W, j = e / W;
    double2 acc = cmk(0.0, 0.0);
    for (int l = 0; l < W; ++l) {
      const double2 a = CA ? cconj(A[i * W + l]) : A[l * W + i];
      const double2 b = CB ? cconj(B[l * W + j]) : B[j * W + l];
      cfma(acc, a, b);
    }
    C[e] = acc;
  }
}

// polar factor U (U^H U)^{-1/2} of a full-rank W x W matrix, in place in U: the unitary
// factor L R of its SVD (orthogonalize_u).  S, V, T: W x W scratch.  Returns false when
// U^H U is not positive definite or the eigensolver did not converge.
__device__ bool sym_polar(double2* U, double2* S, double2* V, double2* T, int W, double* red, double* rc,
                          double2* rse, int* rp, int* rq) {
  const int WW = W * W;
  sym_mm<true, false>(S, U, U, W);
  __syncthreads();
  const int sweeps = cta_jacobi(S, V, W, 60, red, rc, rse, rp, rq);
  __shared__ int bad;
  if (threadIdx.x == 0) bad = sweeps < 0;
  __syncthreads();
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    const int j = e / W;
    const double l = S[j * W + j].x;
    if (!(l > 0.0)) bad = 1;
    T[e] = cscale(V[e], 1.0 / sqrt(l));       // V L^{-1/2}
  }
  __syncthreads();
  sym_mm<false, false>(S, U, T, W);            // U V L^{-1/2}
  __syncthreads();
  sym_mm<false, true>(U, S, V, W);             // ... V^H
  __syncthreads();
  return bad == 0;
}

}  // namespace

// ----------------------------------------------------------------------------
// k_sym_grad: gradient symmetrisation (modes 1 and 2) and the CG partials it changes.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sym_grad(const Problem* __restrict__ probs, WorkMap wm) {
  __shared__ double red[256];
  int ir;
  const int p = locate(wm, blockIdx.x, ir);
  const Problem& P = probs[p];
  const CtrlState* st = P.st;
  if (st->done) return;
  const int W = P.W, WW = W * W;
  const int ik = P.sym_ik[ir];
  double2* Gk = P.G + (size_t)ik * WW;
  double2* Tot = P.sym_work + (size_t)ir * kSymWork * WW;
  double2* A = Tot + WW;
  double2* Bm = Tot + 2 * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) Tot[e] = Gk[e];
  __syncthreads();
  // mode 1: G(k_ir) += D(R,k)^+ G(R k) D(R,k) over the star, in first-occurrence order
  for (int m = P.sym_moff[ir]; m < P.sym_moff[ir + 1]; ++m) {
    const double2* D = P.sym_d + (size_t)P.sym_mem[2 * m + 1] * WW;
    const double2* Gm = P.G + (size_t)P.sym_mem[2 * m] * WW;
    sym_mm<true, false>(A, D, Gm, W);          // cmat2 = D^+ G(Rk)
    __syncthreads();
    sym_mm<false, false>(Bm, A, D, W);         // cmat1 = cmat2 D
    __syncthreads();
    for (int e = threadIdx.x; e < WW; e += blockDim.x) Tot[e] = cadd(Tot[e], Bm[e]);
    __syncthreads();
  }
  // mode 2: average over the little group {R : R k = k} (the identity excluded from the sum)
  const int g0 = P.sym_goff[ir], g1 = P.sym_goff[ir + 1];
  const int ngk = g1 - g0;
  double2* G1 = Tot;
  if (ngk > 1) {
    double2* Tot2 = Tot + 3 * WW;
    for (int e = threadIdx.x; e < WW; e += blockDim.x) Tot2[e] = G1[e];
    __syncthreads();
    for (int g = g0; g < g1; ++g) {
      if (P.sym_grp[2 * g] == 0) continue;     // isym = 1 (the identity)
      const double2* D = P.sym_d + (size_t)P.sym_grp[2 * g + 1] * WW;
      sym_mm<false, false>(A, G1, D, W);       // cmat2 = G D
      __syncthreads();
      sym_mm<true, false>(Bm, D, A, W);        // cmat1 = D^+ cmat2
      __syncthreads();
      for (int e = threadIdx.x; e < WW; e += blockDim.x) Tot2[e] = cadd(Tot2[e], Bm[e]);
      __syncthreads();
    }
    G1 = Tot2;
  }
  const double inv = ngk > 1 ? 1.0 / (double)ngk : 1.0;
  const double2* Dp = P.D + (size_t)ik * WW;
  double g2 = 0.0, gd = 0.0;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    const double2 g = ngk > 1 ? cmk(G1[e].x * inv, G1[e].y * inv) : G1[e];
    Gk[e] = g;
    const double2 d = Dp[e];
    g2 += g.x * g.x + g.y * g.y;
    gd += g.x * d.x + g.y * d.y;
  }
  // the reducible k of the star: zero gradient
  for (int m = P.sym_moff[ir]; m < P.sym_moff[ir + 1]; ++m) {
    double2* Gm = P.G + (size_t)P.sym_mem[2 * m] * WW;
    for (int e = threadIdx.x; e < WW; e += blockDim.x) Gm[e] = cmk(0.0, 0.0);
  }
  g2 = block_sum(g2, red);
  gd = block_sum(gd, red);
  // CG partials in k_grad's layout ([k][tile] pairs): the whole k_ir on its first tile,
  // zero elsewhere in the star
  const int nt = (W + 31) / 32, ntt = nt * nt;
  if (threadIdx.x == 0) {
    P.gpart[(size_t)ik * ntt * 2] = g2;
    P.gpart[(size_t)ik * ntt * 2 + 1] = gd;
  }
  for (int i = threadIdx.x; i < ntt; i += blockDim.x)
    if (i > 0) {
      P.gpart[((size_t)ik * ntt + i) * 2] = 0.0;
      P.gpart[((size_t)ik * ntt + i) * 2 + 1] = 0.0;
    }
  for (int m = P.sym_moff[ir]; m < P.sym_moff[ir + 1]; ++m) {
    const size_t k = (size_t)P.sym_mem[2 * m];
    for (int i = threadIdx.x; i < 2 * ntt; i += blockDim.x) P.gpart[k * ntt * 2 + i] = 0.0;
  }
}

// ----------------------------------------------------------------------------
// k_sym_dir: D = coefG (G or Gp) + coefD D_prev at k_ir (the expression the exp kernels
// use), D(R k) = D(R,k) D(k_ir) D(R,k)^+ over the star.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sym_dir(const Problem* __restrict__ probs, WorkMap wm) {
  int ir;
  const int p = locate(wm, blockIdx.x, ir);
  const Problem& P = probs[p];
  const CtrlState* st = P.st;
  if (st->done) return;
  const int W = P.W, WW = W * W;
  const int ik = P.sym_ik[ir];
  const double cg = st->coefG, cd = st->coefD;
  const double2* Gk = (st->use_gp ? P.pc_gp : P.G) + (size_t)ik * WW;
  double2* Dk = P.D + (size_t)ik * WW;
  double2* A = P.sym_work + (size_t)ir * kSymWork * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) Dk[e] = cadd(cscale(Gk[e], cg), cscale(Dk[e], cd));
  __syncthreads();
  for (int m = P.sym_moff[ir]; m < P.sym_moff[ir + 1]; ++m) {
    const double2* D = P.sym_d + (size_t)P.sym_mem[2 * m + 1] * WW;
    double2* Dm = P.D + (size_t)P.sym_mem[2 * m] * WW;
    sym_mm<false, true>(A, Dk, D, W);          // D(k) D(R,k)^+
    __syncthreads();
    sym_mm<false, false>(Dm, D, A, W);         // D(R,k) ...
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------
// k_sym_u: symmetry-adapted initial U (projection).  status[ir]: 0 ok, 1 symmetrize_ukirr
// not converged in 100 passes, 2 polar factor failed.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sym_u(const Problem* __restrict__ probs, WorkMap wm) {
  __shared__ double red[256];
  __shared__ double rc[128];
  __shared__ double2 rse[128];
  __shared__ int rp[128], rq[128];
  __shared__ int s_done;
  int ir;
  const int p = locate(wm, blockIdx.x, ir);
  const Problem& P = probs[p];
  const int W = P.W, WW = W * W;
  const int ik = P.sym_ik[ir];
  double2* Uk = P.U[P.st->cur] + (size_t)ik * WW;
  // workspace: U, the sum Us, products A and Bm, and C2; the polar factor's scratch
  // (S, V, T) reuses Us, A and Bm once the sum has been taken
  double2* U = P.sym_work + (size_t)ir * kSymWork * WW;
  double2* Us = U + WW;
  double2* A = U + 2 * WW;
  double2* Bm = U + 3 * WW;
  double2* C2 = U + 4 * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) U[e] = Uk[e];
  const int g0 = P.sym_goff[ir], g1 = P.sym_goff[ir + 1];
  const int ngk = g1 - g0;
  int status = 0;
  __syncthreads();
  if (ngk == 1) {
    if (!sym_polar(U, Us, A, Bm, W, red, rc, rse, rp, rq)) status = 2;
  } else {
    for (int it = 1; it <= 100; ++it) {
      // Us = sum_R d(R,k)^+ U D(R,k);  C2 = ngk I - sum_R U^+ d(R,k)^+ U D(R,k)
      for (int e = threadIdx.x; e < WW; e += blockDim.x) {
        Us[e] = cmk(0.0, 0.0);
        C2[e] = cmk((e % W) == (e / W) ? (double)ngk : 0.0, 0.0);
      }
      __syncthreads();
      for (int g = g0; g < g1; ++g) {
        const double2* D = P.sym_d + (size_t)P.sym_grp[2 * g + 1] * WW;
        const double2* d = P.sym_db + (size_t)P.sym_grp[2 * g + 1] * WW;
        sym_mm<false, false>(A, U, D, W);      // cmat_sub = U D
        __syncthreads();
        sym_mm<true, false>(Bm, d, A, W);      // cmat = d^+ cmat_sub
        __syncthreads();
        for (int e = threadIdx.x; e < WW; e += blockDim.x) {
          Us[e] = cadd(Us[e], Bm[e]);
          const int i = e % W, j = e / W;
          double2 acc = cmk(0.0, 0.0);
          for (int l = 0; l < W; ++l) cfmac(acc, U[i * W + l], Bm[j * W + l]);   // (U^+ cmat)_ij
          C2[e] = csub(C2[e], acc);
        }
        __syncthreads();
      }
      double diff = 0.0;
      for (int e = threadIdx.x; e < WW; e += blockDim.x) diff += sqrt(cabs2(C2[e]));
      diff = block_sum(diff, red);
      if (threadIdx.x == 0) s_done = diff < P.sym_eps ? 1 : (it == 100 ? -1 : 0);
      __syncthreads();
      if (s_done == 1) break;
      if (s_done == -1) {
        status = 1;
        break;
      }
      const double inv = 1.0 / (double)ngk;
      for (int e = threadIdx.x; e < WW; e += blockDim.x) U[e] = cscale(Us[e], inv);
      __syncthreads();
      if (!sym_polar(U, Us, A, Bm, W, red, rc, rse, rp, rq)) {
        status = 2;
        break;
      }
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < WW; e += blockDim.x) Uk[e] = U[e];
  __syncthreads();
  // U(R k) = d(R,k) U(k) D(R,k)^+ over the star
  for (int m = P.sym_moff[ir]; m < P.sym_moff[ir + 1]; ++m) {
    const int slot = P.sym_mem[2 * m + 1];
    const double2* D = P.sym_d + (size_t)slot * WW;
    const double2* d = P.sym_db + (size_t)slot * WW;
    double2* Um = P.U[P.st->cur] + (size_t)P.sym_mem[2 * m] * WW;
    sym_mm<false, false>(A, d, U, W);          // cmat = d U
    __syncthreads();
    sym_mm<false, true>(Um, A, D, W);          // cmat D^+
    __syncthreads();
  }
  if (threadIdx.x == 0) P.sym_status[ir] = status;
}

}  // namespace w90g
