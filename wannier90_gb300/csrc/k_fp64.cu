// FP64 kernels of the GB300 MLWF engine (the plain FP64 path).
//
// One iteration of wann_main (src/wannierise.F90:534-816) is the fixed launch sequence
//   k_grad [-> k_precond(0) -> k_precond(1)] -> k_ctrl_search -> k_exp_u(0) -> k_m_update(0) -> spread(0) -> k_ctrl_step
//   -> k_exp_u(1) -> k_m_update(1) -> spread(1) -> k_ctrl_end
// where spread(slot) = k_omega_p1 -> k_omega_p2.
// All data-dependent decisions of the reference (CG reset, uphill reversal, parabolic
// line search, convergence) are taken on the device by the k_ctrl_* kernels, so the
// sequence never needs the host and can be replayed (or graph-captured) blindly:
// kernels whose work is not needed (second update when the parabola was rejected,
// anything after convergence) return at entry.
//
// GB300's FP64 pipe is ~1/64 of its FP32 rate, so these kernels are FP64-issue bound
// for W >= 8; they are written to minimise FP64 instructions (reciprocals of M_nn
// precomputed, exp(X) by an optimised Taylor scheme instead of an eigensolver) and keep
// W <= 32 operands in shared memory.
#include "cta.cuh"

namespace w90g {

constexpr int kSmemW = 32;   // W <= kSmemW: all per-matrix operands live in shared memory

// ----------------------------------------------------------------------------
// CTA-wide helpers
// ----------------------------------------------------------------------------
// C = op(A) * B for W x W column-major matrices (generic pointers: shared or global).
// CA: op(A) = A^H (A read as conj(A[i*lda+l])), else op(A) = A.
// Each thread computes a 2x2 micro-tile of C.  C must not alias A or B.
template <bool CA>
__device__ void cta_gemm(double2* __restrict__ C, int ldc, const double2* __restrict__ A, int lda,
                         const double2* __restrict__ B, int ldb, int W) {
  const int nb = (W + 1) >> 1;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int i0 = (t % nb) * 2, j0 = (t / nb) * 2;
    const bool i1 = (i0 + 1) < W, j1 = (j0 + 1) < W;
    double2 c00 = cmk(0, 0), c01 = cmk(0, 0), c10 = cmk(0, 0), c11 = cmk(0, 0);
    const double2 z = cmk(0, 0);
#pragma unroll 4
    for (int l = 0; l < W; ++l) {
      double2 a0, a1;
      if (CA) {
        a0 = cconj(A[i0 * lda + l]);
        a1 = i1 ? cconj(A[(i0 + 1) * lda + l]) : z;
      } else {
        a0 = A[l * lda + i0];
        a1 = i1 ? A[l * lda + i0 + 1] : z;
      }
      const double2 b0 = B[j0 * ldb + l];
      const double2 b1 = j1 ? B[(j0 + 1) * ldb + l] : z;
      cfma(c00, a0, b0);
      cfma(c10, a1, b0);
      cfma(c01, a0, b1);
      cfma(c11, a1, b1);
    }
    C[j0 * ldc + i0] = c00;
    if (i1) C[j0 * ldc + i0 + 1] = c10;
    if (j1) {
      C[(j0 + 1) * ldc + i0] = c01;
      if (i1) C[(j0 + 1) * ldc + i0 + 1] = c11;
    }
  }
}

// Per-block statistics of one M(k,b): Im ln M_nn, |M_nn|^2, sum_{m!=n}|M_mn|^2.
// (the quantities wann_omega reads, src/wannierise.F90:2034-2043, :2076-2090, :2241-2258)
__device__ void block_stats(const double2* Mb, int ld, int W, double* ln_out, double* abs2_out,
                            double* offd_out, double* red, const Problem* P = nullptr, size_t kb = 0) {
  double off = 0.0;
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
    const int m = e % W, n = e / W;
    const double2 v = Mb[n * ld + m];
    if (m != n) off += cabs2(v);
  }
  for (int n = threadIdx.x; n < W; n += blockDim.x) {
    const double2 d = Mb[n * ld + n];
    ln_out[n] = P ? guided_ln(*P, kb * W + n, d) : atan2(d.y, d.x);
    abs2_out[n] = d.x * d.x + d.y * d.y;
  }
  const double tot = block_sum(off, red);
  if (threadIdx.x == 0) *offd_out = tot;
}

// ----------------------------------------------------------------------------
// k_mdiag: statistics of every block of M[cur] (initial spread, after projection)
// grid: one CTA per (problem, k*B+b), 128 threads
// ----------------------------------------------------------------------------
__global__ void k_mdiag(const Problem* __restrict__ probs, WorkMap wm) {
  __shared__ double red[128];
  int local;
  const int p = locate(wm, blockIdx.x, local);
  const Problem& P = probs[p];
  const int W = P.W;
  const double2* Mb = P.M[P.st->cur] + (size_t)local * W * W;
  block_stats(Mb, W, W, P.diag_ln + (size_t)local * W, P.diag_abs2 + (size_t)local * W,
              P.offd + local, red, &P, (size_t)local);
}

// ----------------------------------------------------------------------------
// wann_omega (src/wannierise.F90:1979-2284) as a deterministic three-pass reduction
// over chunks of kOmegaChunk (k,b) blocks:
//   p1: per chunk  P_n = sum wb b ln_n (3W), q_n = sum wb (1 - |M_nn|^2 + ln_n^2) (W),
//       sum wb offd, and (first pass only) sum wb (W - sum|M|^2)
//   p2: rave = -(1/K) sum_chunks P (same fixed order in every CTA), then the chunk's
//       part of sum wb (ln_n + b.rave_n)^2
//   p3: one CTA per problem: totals, centres, spreads, Omega terms.
// Selective localisation (slwf_num = s > 0, :2144-2211): p1's off-diagonal slot holds
// sum over n < s of wb (1 - |M_nn|^2 + lambda ln_n^2) (Omega_IOD) and its Omega_I slot
// sum over n < s of 2 wb lambda ln_n (b.c_n) (the k-sum of Omega_nu); p2 sums over n < s
// only; p3 forms Omega_D = (1 - lambda) dd / K, Omega_nu = that sum / K + lambda sum |c_n|^2.
// slot: 0 trial, 1 optimal step, 2 initial (accepted).  Fixed thread ownership and
// fixed-order reductions make the result independent of scheduling.
// ----------------------------------------------------------------------------
constexpr int kOmegaChunk = 64;

// Whether this CTA is the last of the problem's nchunk CTAs to finish (all threads get
// the answer).  Every CTA makes its partials visible device-wide before it counts itself
// in; the last one then reads all of them (through L2) and sums them in chunk order, so
// the totals do not depend on which CTA comes last.
__device__ __forceinline__ bool last_chunk_cta(unsigned* arrive, int nchunk) {
  __shared__ int s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(arrive, 1u) == (unsigned)(nchunk - 1));
  __syncthreads();
  const bool last = s_last != 0;
  if (last) __threadfence();
  return last;
}

__device__ __forceinline__ bool omega_skip(const CtrlState* st, int slot) {
  if (slot < 2) {
    if (st->done) return true;
    if (slot == 1 && !st->do_second) return true;
  }
  return false;
}

__global__ void __launch_bounds__(256) k_omega_p1(const Problem* __restrict__ probs, WorkMap wm, int slot) {
  __shared__ double red[256];
  int ch;
  const int p = locate(wm, blockIdx.x, ch);
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (omega_skip(st, slot)) return;
  const int W = P.W, B = P.B;
  const int KB = P.K * B;
  const int kb0 = ch * kOmegaChunk, kb1 = min(KB, kb0 + kOmegaChunk);
  const int t = threadIdx.x;
  const int nsub = blockDim.x / W;           // W <= 256
  const int n = t % W, sub = t / W;
  const bool act = sub < nsub;
  double r0 = 0, r1 = 0, r2 = 0, q = 0;
  // selective localisation: this thread's WF is an objective one
  const bool obj = P.slwf_num > 0 && n < P.slwf_num;
  const double lam = P.slwf_lambda;
  double iod = 0.0, nu = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0;
  if (obj) {
    c0 = P.slwf_c[n];
    c1 = P.slwf_c[W + n];
    c2 = P.slwf_c[2 * W + n];
  }
  if (act) {
    for (int kb = kb0 + sub; kb < kb1; kb += nsub) {
      const double w = P.wb[kb % B];
      const double l = P.diag_ln[(size_t)kb * W + n];
      const double a = P.diag_abs2[(size_t)kb * W + n];
      const double* bv = P.bk + (size_t)kb * 3;
      const double wl = w * l;
      r0 = fma(wl, bv[0], r0);
      r1 = fma(wl, bv[1], r1);
      r2 = fma(wl, bv[2], r2);
      q += w * (1.0 - a + l * l);
      if (obj) {
        const double bc = bv[0] * c0 + bv[1] * c1 + bv[2] * c2;
        iod += w * (1.0 - a + lam * l * l);
        nu += 2.0 * wl * lam * bc;
      }
    }
  }
  double* out = P.opart1 + (size_t)ch * (4 * W + 2);
  const double vals[4] = {r0, r1, r2, q};
  for (int c = 0; c < 4; ++c) {
    red[t] = act ? vals[c] : 0.0;
    __syncthreads();
    if (t < W) {
      double sacc = 0.0;
      for (int u = 0; u < nsub; ++u) sacc += red[u * W + t];
      out[c * W + t] = sacc;
    }
    __syncthreads();
  }
  if (P.slwf_num > 0) {
    // Omega_IOD in the off-diagonal slot, the k-sum of Omega_nu in the Omega_I slot
    iod = block_sum(act ? iod : 0.0, red);
    nu = block_sum(act ? nu : 0.0, red);
    if (t == 0) {
      out[4 * W] = iod;
      out[4 * W + 1] = nu;
    }
  } else {
    const bool first = (slot == 2) && st->first_pass;
    double od = 0.0, oi = 0.0;
    for (int kb = kb0 + t; kb < kb1; kb += blockDim.x) {
      const double w = P.wb[kb % B];
      double o;
      if (P.tensor && slot < 2) {
        // tensor path: |M(k,b)|_F^2 is invariant under the unitary rotation, so the
        // off-diagonal sum is |M0(k,b)|_F^2 minus the diagonal (src/wannierise.F90:2214-2258)
        double sd = 0.0;
        for (int m = 0; m < W; ++m) sd += P.diag_abs2[(size_t)kb * W + m];
        o = P.frob0[kb] - sd;
      } else {
        o = P.offd[kb];
      }
      od += w * o;
      if (first) {
        double sd = 0.0;
        for (int m = 0; m < W; ++m) sd += P.diag_abs2[(size_t)kb * W + m];
        oi += w * ((double)W - (o + sd));
      }
    }
    od = block_sum(od, red);
    oi = block_sum(oi, red);
    if (t == 0) {
      out[4 * W] = od;
      out[4 * W + 1] = oi;
    }
  }
  if (!last_chunk_cta(&st->omega_arrive[0], P.nchunk)) return;
  // ---- the last CTA: every chunk sum in chunk order on its own thread -- rave (3W) into
  // the slot's centres, r^2 (W) into its spreads, the Omega_OD and Omega_I totals (2)
  double* cen = P.centres + (size_t)slot * 4 * W;
  const int stride = 4 * W + 2;
  __shared__ double s_rave[3 * 256];
  __shared__ double s_q[256];
  for (int i = t; i < 4 * W + 2; i += blockDim.x) {
    double sacc = 0.0;
    for (int c = 0; c < P.nchunk; ++c) sacc += __ldcg(P.opart1 + (size_t)c * stride + i);
    if (i < 3 * W) s_rave[i] = -sacc / (double)P.K;
    else if (i < 4 * W) s_q[i - 3 * W] = sacc;
    else st->omega_tot[i - 4 * W] = sacc;
  }
  __syncthreads();
  for (int i = t; i < W; i += blockDim.x) {
    const double x0 = s_rave[i], x1 = s_rave[W + i], x2 = s_rave[2 * W + i];
    cen[i] = x0;
    cen[W + i] = x1;
    cen[2 * W + i] = x2;
    cen[3 * W + i] = s_q[i] / (double)P.K - (x0 * x0 + x1 * x1 + x2 * x2);
  }
  if (t == 0) st->omega_arrive[0] = 0u;
}

__global__ void __launch_bounds__(256) k_omega_p2(const Problem* __restrict__ probs, WorkMap wm, int slot) {
  __shared__ double red[256];
  int ch;
  const int p = locate(wm, blockIdx.x, ch);
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (omega_skip(st, slot)) return;
  const int W = P.W, B = P.B, K = P.K;
  const int KB = K * B;
  const int kb0 = ch * kOmegaChunk, kb1 = min(KB, kb0 + kOmegaChunk);
  const int t = threadIdx.x;
  const int nsub = blockDim.x / W;
  const int n = t % W, sub = t / W;
  // rave from pass 1's last CTA (the slot's centres)
  const double* cen = P.centres + (size_t)slot * 4 * W;
  double dd = 0.0;
  // selective localisation: Omega_D over the objective WFs only
  if (sub < nsub && (P.slwf_num == 0 || n < P.slwf_num)) {
    const double x0 = cen[n], x1 = cen[W + n], x2 = cen[2 * W + n];
    for (int kb = kb0 + sub; kb < kb1; kb += nsub) {
      const double w = P.wb[kb % B];
      const double* bv = P.bk + (size_t)kb * 3;
      const double l = P.diag_ln[(size_t)kb * W + n] + (bv[0] * x0 + bv[1] * x1 + bv[2] * x2);
      dd = fma(w * l, l, dd);
    }
  }
  dd = block_sum(dd, red);
  if (t == 0) P.opart2[ch] = dd;
  if (!last_chunk_cta(&st->omega_arrive[1], P.nchunk)) return;
  // ---- the last CTA: the Omega_D total in chunk order, then the spread of the slot
  if (t == 0) {
    double acc = 0.0;
    for (int c = 0; c < P.nchunk; ++c) acc += __ldcg(P.opart2 + c);
    const double od = st->omega_tot[0], oi = st->omega_tot[1], dsum = acc;
    Spread sp;
    if (P.slwf_num > 0) {
      // Omega_tot = Omega_IOD + Omega_D + Omega_nu (Omega_I is never formed); om_od
      // carries Omega_IOD + Omega_nu, what the reference prints as O_IOD
      const double iod = od / (double)K;
      sp.om_nu = oi / (double)K + P.slwf_nu0;
      sp.om_i = 0.0;
      sp.om_d = (1.0 - P.slwf_lambda) * dsum / (double)K;
      sp.om_od = iod + sp.om_nu;
      sp.om_tot = iod + sp.om_d + sp.om_nu;
    } else {
      if ((slot == 2) && st->first_pass) {
        st->om_invariant = oi / (double)K;
        st->first_pass = 0;
      }
      sp.om_i = st->om_invariant;
      sp.om_d = dsum / (double)K;
      sp.om_od = od / (double)K;
      sp.om_tot = sp.om_i + sp.om_d + sp.om_od;
      sp.om_nu = 0.0;
    }
    if (slot == 2) st->wann = sp;
    else st->slot[slot] = sp;
    if (!isfinite(sp.om_tot)) {
      st->error = 1;
      st->done = 1;
    }
    st->omega_arrive[1] = 0u;
  }
}

// ----------------------------------------------------------------------------
// k_grad: wann_domega (src/wannierise.F90:2287-2569), both branches, fused with the
// per-k partial dot products of internal_search_direction (:1424-1431).
// rave is the one computed by the preceding spread pass on the same M (the reference
// recomputes it from the same data, :2378-2393).
// ----------------------------------------------------------------------------
constexpr int kTile = 32;

// Im ln M_nn(k,b) of the accepted M for the gradient: the block statistics already hold it
// (written from the same M_nn by the pass that formed M, with the same function), except
// with guiding centres, whose sheets may have moved since (k_phases runs first)
__device__ __forceinline__ double diag_ln_of(const Problem& P, size_t kbn, double2 d) {
  return P.guiding ? guided_ln(P, kbn, d) : P.diag_ln[kbn];
}

// q of the factored gradient for index j (row or column) of block (k,b): the plain form
// wb (ln_j + b.r_j) for both variants; with selective localisation (src/wannierise.F90:
// 2431-2509, factored) qx for a partner inside the objective block and qy for one outside
//   qx = wb ln_j + (b.r_j)(1 - wb lambda) + wb lambda (b.c_j)
//   qy = wb ln_j + wb (b.r_j)(1 - lambda) + wb lambda (b.c_j)
// and false for a non-objective j, whose coefficients are zero.
__device__ __forceinline__ bool grad_q(const Problem& P, double w, double l, double brn, const double* bv, int j,
                                       double& qx, double& qy) {
  if (P.slwf_num == 0) {
    qx = qy = w * (l + brn);
    return true;
  }
  if (j >= P.slwf_num) return false;
  const double lam = P.slwf_lambda;
  const int W = P.W;
  const double r0 = bv[0] * P.slwf_c[j] + bv[1] * P.slwf_c[W + j] + bv[2] * P.slwf_c[2 * W + j];
  qx = w * l + brn * (1.0 - w * lam) + w * lam * r0;
  qy = w * l + w * brn * (1.0 - lam) + w * lam * r0;
  return true;
}

// The gradient is anti-Hermitian, and the reference forms it exactly so: every term of
// wann_domega is X - X^H of one (k,b) block (:2518-2527).  With
//   alpha_n = wb/2 conj(M_nn) + (i/2) q_n / M_nn      (q_n from grad_q)
// that sum is G = (4/K)(P - P^H),  P_mn = sum_b M_mn(k,b) alpha^{v(m)}_n(k,b),
// where the variant v(m) selects q by the partner index m (inside / outside the objective
// block; one variant without selective localisation).  So one complex FMA per element
// and b, all reads coalesced down columns; the transpose happens once, in shared memory.
// Grid: one CTA per (problem, k, ti, tj) of 32 x 32 tiles, 256 threads.  The CTA with
// ti <= tj forms P over tiles (ti,tj) and (tj,ti) (one tile when ti == tj) and writes
// G on both; a CTA with ti > tj only clears its partial slots.
constexpr int kGradBC = 8;   // b values whose coefficients are staged together

__global__ void __launch_bounds__(256) k_grad(const Problem* __restrict__ probs, WorkMap wm) {
  __shared__ double2 s_alpha[2][kGradBC][kTile];
  __shared__ double2 sP[2][kTile * (kTile + 1)];   // sP[t][j*(33)+i]: P tile t, row i, column j
  __shared__ double red[256];
  int local;
  const int p = locate(wm, blockIdx.x, local);
  const Problem& P = probs[p];
  const CtrlState* st = P.st;
  if (st->done) return;
  const int W = P.W, B = P.B, K = P.K;
  const int nt = (W + kTile - 1) / kTile;
  const int k = local / (nt * nt);
  const int tt = local % (nt * nt);
  const int ti = tt % nt, tj = tt / nt;
  const int t = threadIdx.x;
  if (ti > tj) {
    if (t == 0) {
      P.gpart[(size_t)local * 2] = 0.0;
      P.gpart[(size_t)local * 2 + 1] = 0.0;
    }
    return;
  }
  const double* rave = P.centres + (size_t)2 * 4 * W;  // accepted slot
  const double2* __restrict__ Mk = P.M[st->cur] + (size_t)k * B * W * W;
  const int S = P.slwf_num > 0 ? P.slwf_num : W;   // objective WFs 0..S-1
  const int npass = (ti == tj) ? 1 : 2;
  for (int pass = 0; pass < npass; ++pass) {
    // P tile `pass`: rows R0.., columns C0..  (pass 0: (ti,tj); pass 1: (tj,ti))
    const int R0 = (pass == 0 ? ti : tj) * kTile, C0 = (pass == 0 ? tj : ti) * kTile;
    const int nr = min(kTile, W - R0), nc = min(kTile, W - C0);
    double2 acc[4];
    int vrow[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      acc[q] = cmk(0, 0);
      const int i = (t + 256 * q) % kTile;
      vrow[q] = (R0 + i < S) ? 0 : 1;
    }
    for (int b0 = 0; b0 < B; b0 += kGradBC) {
      const int nb = min(kGradBC, B - b0);
      __syncthreads();   // the previous chunk's coefficients are consumed
      // coefficients of the chunk: thread (bl, u) for column n = C0 + u of block b0 + bl
      {
        const int bl = t / kTile, u = t % kTile;
        if (bl < nb && u < nc) {
          const int b = b0 + bl, n = C0 + u;
          const double w = P.wb[b];
          const double* bv = P.bk + ((size_t)k * B + b) * 3;
          const double2 d = Mk[((size_t)b * W + n) * W + n];
          const double inv = 1.0 / (d.x * d.x + d.y * d.y);
          const double brn = bv[0] * rave[n] + bv[1] * rave[W + n] + bv[2] * rave[2 * W + n];
          double qv[2];
          if (grad_q(P, w, diag_ln_of(P, ((size_t)k * B + b) * W + n, d), brn, bv, n, qv[0], qv[1])) {
            // 1/M_nn = (d.x - i d.y) inv ;  (i/2) q / M_nn = (q inv / 2)(d.y + i d.x)
            for (int v = 0; v < 2; ++v)
              s_alpha[v][bl][u] = cmk(0.5 * w * d.x + 0.5 * qv[v] * inv * d.y, -0.5 * w * d.y + 0.5 * qv[v] * inv * d.x);
          } else {
            s_alpha[0][bl][u] = s_alpha[1][bl][u] = cmk(0.0, 0.0);
          }
        }
      }
      __syncthreads();
      // P_mn += M_mn alpha^{v(m)}_n; four b blocks' loads issued together
#pragma unroll 4
      for (int bl = 0; bl < nb; ++bl) {
        const double2* Mb = Mk + (size_t)(b0 + bl) * W * W;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int e = t + 256 * q;
          const int i = e % kTile, j = e / kTile;
          if (i < nr && j < nc) cfma(acc[q], Mb[(size_t)(C0 + j) * W + R0 + i], s_alpha[vrow[q]][bl][j]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = t + 256 * q;
      sP[pass][(e / kTile) * (kTile + 1) + e % kTile] = acc[q];
    }
  }
  __syncthreads();
  // G = fac (P - P^H) on tile (ti,tj) and, off the diagonal, on tile (tj,ti):
  // G_mn = fac (P_mn - conj(P_nm)); the mirrored element is the exact -conj of it
  const double fac = 4.0 / (double)K;
  double g2 = 0.0, gd = 0.0;
  double2* Gk = P.G + (size_t)k * W * W;
  const double2* Dk = P.D + (size_t)k * W * W;
  const int other = npass - 1;   // sP index of the transposed tile
  for (int pass = 0; pass < npass; ++pass) {
    const int R0 = (pass == 0 ? ti : tj) * kTile, C0 = (pass == 0 ? tj : ti) * kTile;
    const int nr = min(kTile, W - R0), nc = min(kTile, W - C0);
    const double2* mine = sP[pass == 0 ? 0 : 1];
    const double2* tr = sP[pass == 0 ? other : 0];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = t + 256 * q;
      const int i = e % kTile, j = e / kTile;
      if (i < nr && j < nc) {
        const double2 a = mine[j * (kTile + 1) + i];
        const double2 c = tr[i * (kTile + 1) + j];   // P_nm: row j, column i of the transposed tile
        const double2 g = cmk(fac * (a.x - c.x), fac * (a.y + c.y));
        const size_t off = (size_t)(C0 + j) * W + R0 + i;
        Gk[off] = g;
        const double2 d = Dk[off];
        g2 += g.x * g.x + g.y * g.y;
        gd += g.x * d.x + g.y * d.y;
      }
    }
  }
  g2 = block_sum(g2, red);
  gd = block_sum(gd, red);
  if (t == 0) {
    P.gpart[(size_t)local * 2] = g2;
    P.gpart[(size_t)local * 2 + 1] = gd;
  }
}

// ----------------------------------------------------------------------------
// k_phases: wann_phases (src/wannierise.F90:1756-1976) for guiding centres.
// mode 0: before the loop (num_no_guide_iter <= 0, centres not refitted);
// mode 1: at the start of an iteration with iter > num_no_guide_iter and
// mod(iter, num_guide_cycles) = 0.  One CTA per (n, problem):
//   csum_a = sum_k M_nn(k, neigh(k,a)) over the b directions a; the centre is refitted
//   (when irguide != 0) by least squares on the unwrapped phases (:1878-1925); then
//   sheet(n,b,k) = b . rguide_n, csheet = exp(i sheet) and, in mode 1, rave_n on the new
//   branch (what wann_domega recomputes, :2366-2391) for the gradient.
// ----------------------------------------------------------------------------
__global__ void k_phases(const Problem* __restrict__ probs, int mode) {
  __shared__ double red[256];
  __shared__ double s_csum[2 * 8];
  __shared__ double s_rg[3];
  const Problem& P = probs[blockIdx.y];
  const CtrlState* st = P.st;
  const int n = blockIdx.x;
  if (!P.guiding || n >= P.W || st->done) return;
  const int iter = st->iter + 1;
  if (mode == 0 && P.no_guide_iter > 0) return;
  if (mode == 1 && !(iter > P.no_guide_iter && (P.guide_cycles <= 0 || iter % P.guide_cycles == 0))) return;
  const int W = P.W, B = P.B, K = P.K, nnh = P.nnh;
  const double2* M = P.M[st->cur];
  for (int a = 0; a < nnh; ++a) {
    double cr = 0.0, ci = 0.0;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      const int b = P.neigh[(size_t)k * nnh + a];
      const double2 d = M[((size_t)k * B + b) * W * W + (size_t)n * W + n];
      cr += d.x;
      ci += d.y;
    }
    cr = block_sum(cr, red);
    ci = block_sum(ci, red);
    if (threadIdx.x == 0) {
      s_csum[2 * a] = cr;
      s_csum[2 * a + 1] = ci;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double rg[3] = {P.rguide[n], P.rguide[W + n], P.rguide[2 * W + n]};
    double smat[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, svec[3] = {0, 0, 0};
    for (int a = 0; a < nnh; ++a) {
      const double* ba = P.bka + 3 * a;
      const double2 cs = cmk(s_csum[2 * a], s_csum[2 * a + 1]);
      double xx;
      if (a < 3) {
        xx = -atan2(cs.y, cs.x);
      } else {
        const double xx0 = ba[0] * rg[0] + ba[1] * rg[1] + ba[2] * rg[2];
        double sn, cn;
        sincos(xx0, &sn, &cn);
        const double2 z = cmul(cs, cmk(cn, sn));
        xx = xx0 - atan2(z.y, z.x);
      }
      for (int j = 0; j < 3; ++j) {
        for (int i = 0; i < 3; ++i) smat[j][i] += ba[j] * ba[i];
        svec[j] += ba[j] * xx;
      }
      if (a >= 2) {
        // cofactor matrix and determinant (utility_inv3, src/utility.F90:233-262)
        double c[3][3];
        c[0][0] = smat[1][1] * smat[2][2] - smat[2][1] * smat[1][2];
        c[0][1] = smat[1][2] * smat[2][0] - smat[2][2] * smat[1][0];
        c[0][2] = smat[1][0] * smat[2][1] - smat[2][0] * smat[1][1];
        c[1][0] = smat[2][1] * smat[0][2] - smat[0][1] * smat[2][2];
        c[1][1] = smat[2][2] * smat[0][0] - smat[0][2] * smat[2][0];
        c[1][2] = smat[2][0] * smat[0][1] - smat[0][0] * smat[2][1];
        c[2][0] = smat[0][1] * smat[1][2] - smat[1][1] * smat[0][2];
        c[2][1] = smat[0][2] * smat[1][0] - smat[1][2] * smat[0][0];
        c[2][2] = smat[0][0] * smat[1][1] - smat[1][0] * smat[0][1];
        const double det = smat[0][0] * c[0][0] + smat[0][1] * c[0][1] + smat[0][2] * c[0][2];
        if (fabs(det) > 1e-6 && st->irguide != 0) {
          for (int j = 0; j < 3; ++j) {
            double v = 0.0;
            for (int i = 0; i < 3; ++i) v += c[j][i] * svec[i] / det;
            rg[j] = v;
          }
        }
      }
    }
    for (int j = 0; j < 3; ++j) {
      P.rguide[j * W + n] = rg[j];
      s_rg[j] = rg[j];
    }
  }
  __syncthreads();
  const double rg0 = s_rg[0], rg1 = s_rg[1], rg2 = s_rg[2];
  double r0 = 0.0, r1 = 0.0, r2 = 0.0;
  for (int kb = threadIdx.x; kb < K * B; kb += blockDim.x) {
    const double* bv = P.bk + (size_t)kb * 3;
    const double sh = bv[0] * rg0 + bv[1] * rg1 + bv[2] * rg2;
    double sn, cn;
    sincos(sh, &sn, &cn);
    const size_t kbn = (size_t)kb * W + n;
    P.sheet[kbn] = sh;
    P.csheet[kbn] = cmk(cn, sn);
    if (mode == 1) {
      const double2 d = M[(size_t)kb * W * W + (size_t)n * W + n];
      const double2 z = cmul(cmk(cn, sn), d);
      const double ln = atan2(z.y, z.x) - sh;
      const double wl = P.wb[kb % B] * ln;
      r0 += wl * bv[0];
      r1 += wl * bv[1];
      r2 += wl * bv[2];
    }
  }
  if (mode == 1) {
    r0 = block_sum(r0, red);
    r1 = block_sum(r1, red);
    r2 = block_sum(r2, red);
    if (threadIdx.x == 0) {
      // rave of the accepted state on the new branch, read by k_grad
      double* rave = P.centres + (size_t)2 * 4 * W;
      rave[n] = -r0 / K;
      rave[W + n] = -r1 / K;
      rave[2 * W + n] = -r2 / K;
    }
  }
}

// ----------------------------------------------------------------------------
// k_precond: precond_search_direction (src/wannierise.F90:1256-1368), its GEMM form
// (optimisation >= 3, :1314-1320 and :1345-1352):
//   dir 0:  Gr(R) = sum_k G(k) exp(-i 2pi k.R)                          (k -> R)
//   dir 1:  Gp(k) = sum_R f_R Gr(R) exp(+i 2pi k.R),
//           f_R = 1 / (num_kpts * ndegen_R * (1 + |R|^2 / alpha)),  alpha = 10 Omega / W
// Each is a complex GEMM (W^2 x n_out x n_red).  Tile: 64 matrix elements x 16 outputs
// per CTA (256 threads, 4 outputs each), reduction in chunks of 16 through shared memory.
// dir 1 also writes the tile's partial of Re <Gp, G> (gcnorm1 of :1426-1428).
// grid: (CTAs per problem, problems); CTAs beyond a problem's tile count return.
// ----------------------------------------------------------------------------
constexpr int kPcE = 64, kPcO = 16, kPcC = 16;

__global__ void __launch_bounds__(256) k_precond(const Problem* __restrict__ probs, int dir) {
  __shared__ double2 sX[kPcC][kPcE];
  __shared__ double2 sP[kPcC][kPcO];
  __shared__ double sf[kPcC];
  __shared__ double red[256];
  const Problem& P = probs[blockIdx.y];
  const CtrlState* st = P.st;
  if (!P.precond || st->done) return;
  const int WW = P.W * P.W, K = P.K, NR = P.nrpts;
  const int n_out = dir == 0 ? NR : K;
  const int n_red = dir == 0 ? K : NR;
  const int te = (WW + kPcE - 1) / kPcE;
  const int to = (n_out + kPcO - 1) / kPcO;
  const int local = blockIdx.x;
  if (local >= te * to) return;
  const int e0 = (local % te) * kPcE, o0 = (local / te) * kPcO;
  const int t = threadIdx.x;
  const int e = t % kPcE, og = (t / kPcE) * 4;
  const double2* X = dir == 0 ? P.G : P.pc_gr;
  const double alpha = 10.0 * st->wann.om_tot / (double)P.W;
  double2 acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = cmk(0, 0);
  for (int c0 = 0; c0 < n_red; c0 += kPcC) {
    __syncthreads();
    if (dir == 1 && t < kPcC) {
      const int r = c0 + t;
      sf[t] = r < NR ? 1.0 / ((double)K * P.pc_ndeg[r] * (1.0 + P.pc_r2[r] / alpha)) : 0.0;
    }
    for (int i = t; i < kPcC * kPcO; i += 256) {
      const int j = i / kPcO, o = i % kPcO;
      double2 v = cmk(0, 0);
      if (c0 + j < n_red && o0 + o < n_out) {
        v = dir == 0 ? P.pc_kr[(size_t)(c0 + j) * NR + o0 + o]
                     : cconj(P.pc_kr[(size_t)(o0 + o) * NR + c0 + j]);
      }
      sP[j][o] = v;
    }
    __syncthreads();
    for (int i = t; i < kPcC * kPcE; i += 256) {
      const int j = i / kPcE, ee = i % kPcE;
      double2 v = cmk(0, 0);
      if (c0 + j < n_red && e0 + ee < WW) {
        v = X[(size_t)(c0 + j) * WW + e0 + ee];
        if (dir == 1) v = cscale(v, sf[j]);
      }
      sX[j][ee] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < kPcC; ++j) {
      const double2 x = sX[j][e];
#pragma unroll
      for (int q = 0; q < 4; ++q) cfma(acc[q], x, sP[j][og + q]);
    }
  }
  double part = 0.0;
  if (e0 + e < WW) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int o = o0 + og + q;
      if (o >= n_out) continue;
      if (dir == 0) {
        // the 1/num_kpts of :1320 is folded into f_R
        P.pc_gr[(size_t)o * WW + e0 + e] = acc[q];
      } else {
        const size_t off = (size_t)o * WW + e0 + e;
        P.pc_gp[off] = acc[q];
        const double2 g = P.G[off];
        part += acc[q].x * g.x + acc[q].y * g.y;
      }
    }
  }
  if (dir == 1) {
    part = block_sum(part, red);
    if (t == 0) P.pc_part[local] = part;
  }
}

// ----------------------------------------------------------------------------
// k_ctrl_search: internal_search_direction (src/wannierise.F90:1371-1525) as scalars.
// D = G + gcfac*D_prev is never formed here: the coefficients (coefG, coefD) are
// handed to k_exp_u, and <G,D> = |G|^2 + gcfac*<G,D_prev> comes from k_grad's partials.
// One CTA (256 threads) per problem.
// ----------------------------------------------------------------------------
__global__ void k_ctrl_search(const Problem* __restrict__ probs) {
  __shared__ double red[256];
  const Problem& P = probs[blockIdx.x];
  CtrlState* st = P.st;
  if (st->done) return;
  const int nt = (P.W + kTile - 1) / kTile;
  const int n = P.K * nt * nt;
  double g2 = 0.0, gd = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    g2 += P.gpart[(size_t)i * 2];
    gd += P.gpart[(size_t)i * 2 + 1];
  }
  g2 = block_sum(g2, red);
  gd = block_sum(gd, red);
  // precond: gcnorm1 = Re <Gp, G> (:1426-1428) from k_precond's partials
  double gpg = g2;
  if (P.precond) {
    const int te = (P.W * P.W + kPcE - 1) / kPcE;
    const int np = te * ((P.K + kPcO - 1) / kPcO);
    double a = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) a += P.pc_part[i];
    gpg = block_sum(a, red);
  }
  if (threadIdx.x != 0) return;
  const Control& c = P.ctl;
  const int iter = st->iter + 1;
  const double gcnorm1 = gpg;
  double gcfac;
  int ncg = st->ncg;
  if (iter == 1 || ncg >= c.num_cg_steps) {
    gcfac = 0.0;
    ncg = 0;
  } else {
    if (st->gcnorm0 > 2.220446049250313e-16) {   // epsilon(1.0_dp)
      gcfac = gcnorm1 / st->gcnorm0;
      if (gcfac > 3.0) {
        gcfac = 0.0;
        ncg = 0;
      } else {
        ncg = ncg + 1;
      }
    } else {
      gcfac = 0.0;
      ncg = 0;
    }
  }
  st->gcnorm0 = gcnorm1;
  st->gcnorm1 = gcnorm1;
  const double fw = 4.0 * P.wbtot;
  // D = (Gp or G) + gcfac D_prev; <G, Gp> = gcnorm1 (:1460-1464, :1475-1481)
  double coefG = 1.0, coefD = gcfac;
  int use_gp = P.precond;
  double doda0 = -(gpg + gcfac * gd) / fw;
  if (doda0 > 0.0) {
    if (ncg > 0) {
      // reset to the plain gradient, also under precond (:1488)
      coefD = 0.0;
      use_gp = 0;
      ncg = 0;
      gcfac = 0.0;
      doda0 = -g2 / fw;
      if (doda0 > 0.0) {
        coefG = -coefG;
        doda0 = -doda0;
      }
    } else {
      coefG = -coefG;
      coefD = -coefD;
      doda0 = -doda0;
    }
  }
  st->ncg = ncg;
  st->gcfac = gcfac;
  st->doda0 = doda0;
  st->coefG = coefG;
  st->coefD = coefD;
  st->use_gp = use_gp;
  if (P.guiding && iter > P.no_guide_iter && (P.guide_cycles <= 0 || iter % P.guide_cycles == 0)) st->irguide = 1;
  if (c.lfixstep) {
    st->alphamin = c.fixed_step;
    st->s_trial = c.fixed_step / fw;
  } else {
    st->s_trial = c.trial_step / fw;
  }
  st->do_second = 0;
}

// ----------------------------------------------------------------------------
// C = A * B where the product is known to be Hermitian (sign = +1) or anti-Hermitian
// (sign = -1): only the upper-triangular 2x2 tiles are computed (whole warps skip the
// rest), then the lower triangle is mirrored.  Caller synchronises before reading C.
// ----------------------------------------------------------------------------
__device__ void cta_gemm_sym(double2* __restrict__ C, const double2* __restrict__ A,
                             const double2* __restrict__ B, int W, double sign) {
  const int nb = (W + 1) >> 1;
  const int ntri = nb * (nb + 1) / 2;
  for (int t = threadIdx.x; t < ntri; t += blockDim.x) {
    int bi = 0, rem = t;
    while (rem >= nb - bi) {
      rem -= nb - bi;
      ++bi;
    }
    const int bj = bi + rem;
    const int i0 = bi * 2, j0 = bj * 2;
    const bool i1 = (i0 + 1) < W, j1 = (j0 + 1) < W;
    double2 c00 = cmk(0, 0), c01 = cmk(0, 0), c10 = cmk(0, 0), c11 = cmk(0, 0);
    const double2 z = cmk(0, 0);
#pragma unroll 4
    for (int l = 0; l < W; ++l) {
      const double2 a0 = A[l * W + i0];
      const double2 a1 = i1 ? A[l * W + i0 + 1] : z;
      const double2 b0 = B[j0 * W + l];
      const double2 b1 = j1 ? B[(j0 + 1) * W + l] : z;
      cfma(c00, a0, b0);
      cfma(c10, a1, b0);
      cfma(c01, a0, b1);
      cfma(c11, a1, b1);
    }
    C[j0 * W + i0] = c00;
    if (i1) C[j0 * W + i0 + 1] = c10;
    if (j1) {
      C[(j0 + 1) * W + i0] = c01;
      if (i1) C[(j0 + 1) * W + i0 + 1] = c11;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
    const int i = e % W, j = e / W;
    if (i > j) {
      const double2 u = C[i * W + j];   // C(j,i), upper triangle
      C[e] = cmk(sign * u.x, -sign * u.y);
    } else if (i == j) {
      const double2 d = C[e];
      C[e] = (sign > 0) ? cmk(d.x, 0.0) : cmk(0.0, d.y);
    }
  }
}

// ----------------------------------------------------------------------------
// exp(X) for anti-Hermitian X (W x W): scaling and squaring with a Taylor polynomial
// of degree m evaluated by Paterson-Stockmeyer in powers up to X^p.  Per matrix the
// cheapest (m, squarings j) is chosen such that ||X / 2^j||_1 <= theta_m, where
// theta_m^(m+1) / (m+1)! <= 2^-53 bounds the truncation (||e^Y||_2 = 1 for
// anti-Hermitian Y):  (m, p, theta_m, cost in W^3 products) =
//   (4,4,1.6e-3,1.5) (6,3,1.7e-2,2.0) (8,4,6.6e-2,2.5) (12,4,0.32,3.5) (16,4,0.78,4.5)
// X^2 and X^4 are Hermitian and X^3 anti-Hermitian, so those powers cost half a
// product.  exp(s*D) equals the reference's V e^{-i s lambda} V^dagger with (V, lambda)
// the eigenpairs of i*D (src/wannierise.F90:1655-1690) in exact arithmetic.
// Buffers: X (input, scaled in place), Y2, Y3, Y4, R, T (6 * W*W).  Returns the result.
// ----------------------------------------------------------------------------
__device__ const double kInvFact[17] = {
    1.0, 1.0, 0.5, 1.6666666666666666e-01, 4.1666666666666664e-02, 8.3333333333333332e-03,
    1.3888888888888889e-03, 1.9841269841269841e-04, 2.4801587301587302e-05,
    2.7557319223985893e-06, 2.7557319223985888e-07, 2.5052108385441720e-08,
    2.0876756987868100e-09, 1.6059043836821613e-10, 1.1470745597729725e-11,
    7.6471637318198164e-13, 4.7794773323873853e-14};

__device__ double2* cta_expm(double2* X, double2* Y2, double2* Y3, double2* Y4, double2* R,
                             double2* T, int W, double* red, double* cost_out) {
  const int WW = W * W;
  double colmax = 0.0;
  for (int j = threadIdx.x; j < W; j += blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < W; ++i) s += sqrt(cabs2(X[j * W + i]));
    colmax = fmax(colmax, s);
  }
  const double nrm = block_max(colmax, red);
  // candidate degrees (theta_m with a 5% margin for the tail of the series)
  const int cand_m[5] = {4, 6, 8, 12, 16};
  const int cand_p[5] = {4, 3, 4, 4, 4};
  const double cand_theta[5] = {1.6e-3, 1.68e-2, 6.6e-2, 0.32, 0.78};
  const double cand_cost[5] = {1.5, 2.0, 2.5, 3.5, 4.5};
  int m = 16, p = 4, js = 0;
  double best = 1e300;
  for (int c = 0; c < 5; ++c) {
    int j = 0;
    double v = nrm;
    while (v > cand_theta[c] && j < 60) {
      v *= 0.5;
      ++j;
    }
    const double cost = cand_cost[c] + j;
    if (cost < best) {
      best = cost;
      m = cand_m[c];
      p = cand_p[c];
      js = j;
    }
  }
  *cost_out = best;
  const double sc = ldexp(1.0, -js);
  for (int e = threadIdx.x; e < WW; e += blockDim.x) X[e] = cscale(X[e], sc);
  __syncthreads();
  // powers: Y2 Hermitian, Y3 = Y2 X anti-Hermitian, Y4 = Y2 Y2 Hermitian
  cta_gemm_sym(Y2, X, X, W, 1.0);
  __syncthreads();
  cta_gemm_sym(Y3, Y2, X, W, -1.0);
  if (p >= 4) cta_gemm_sym(Y4, Y2, Y2, W, 1.0);
  __syncthreads();
  const double2* Yp = (p == 4) ? Y4 : Y3;
  const int nblk = (m + p) / p;   // blocks B_0 .. B_{nblk-1}, B_q = sum_r c_{pq+r} Y^r
  // element e of B_q
  auto blk = [&](int q, int e) -> double2 {
    const int i = e % W, j = e / W;
    double2 v = cmk(0.0, 0.0);
    for (int r = 0; r < p; ++r) {
      const int deg = p * q + r;
      if (deg > m) break;
      const double c = kInvFact[deg];
      if (r == 0) {
        if (i == j) v.x += c;
      } else {
        const double2 y = (r == 1) ? X[e] : ((r == 2) ? Y2[e] : Y3[e]);
        v = cadd(v, cscale(y, c));
      }
    }
    return v;
  };
  int q = nblk - 1;
  // R = B_top; when B_top is c_m I alone, fold the first Horner step into a scaled copy
  if (p * q == m) {
    const double cm = kInvFact[m];
    for (int e = threadIdx.x; e < WW; e += blockDim.x) R[e] = cadd(cscale(Yp[e], cm), blk(q - 1, e));
    q -= 1;
  } else {
    for (int e = threadIdx.x; e < WW; e += blockDim.x) R[e] = blk(q, e);
  }
  __syncthreads();
  for (q = q - 1; q >= 0; --q) {
    cta_gemm<false>(T, W, Yp, W, R, W, W);
    __syncthreads();
    for (int e = threadIdx.x; e < WW; e += blockDim.x) R[e] = cadd(T[e], blk(q, e));
    __syncthreads();
  }
  double2* a = R;
  double2* b = T;
  for (int s = 0; s < js; ++s) {
    cta_gemm<false>(b, W, a, W, a, W, W);
    __syncthreads();
    double2* tmp = a;
    a = b;
    b = tmp;
  }
  return a;
}

// ----------------------------------------------------------------------------
// k_exp_u: one CTA per (problem, k).  which = 0: trial step (also forms D),
// which = 1: optimal step.  dU(k) = exp(s*D(k));  U[cur^1](k) = U[cur](k) dU(k)
// (src/wannierise.F90:1655-1733).
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_exp_u(const Problem* __restrict__ probs, WorkMap wm, int which) {
  extern __shared__ double2 smem[];
  __shared__ double red[256];
  int k;
  const int p = locate(wm, blockIdx.x, k);
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (st->done) return;
  if (which == 1 && !st->do_second) return;
  const int W = P.W, WW = W * W;
  double2* buf = (W <= kSmemW) ? smem : (P.work + (size_t)k * 6 * WW);
  double2 *X = buf, *Y2 = buf + WW, *Y3 = buf + 2 * WW, *Y4 = buf + 3 * WW, *R = buf + 4 * WW,
          *T = buf + 5 * WW;
  double2* Dk = P.D + (size_t)k * WW;
  const double s = (which == 0) ? st->s_trial : st->s_second;
  if (which == 0 && P.sym_nir == 0) {
    // (in the symmetry-adapted mode k_sym_dir has formed D already)
    const double cg = st->coefG, cd = st->coefD;
    const double2* Gk = (st->use_gp ? P.pc_gp : P.G) + (size_t)k * WW;
    for (int e = threadIdx.x; e < WW; e += blockDim.x) {
      const double2 d = cadd(cscale(Gk[e], cg), cscale(Dk[e], cd));
      Dk[e] = d;
      X[e] = cscale(d, s);
    }
  } else {
    for (int e = threadIdx.x; e < WW; e += blockDim.x) X[e] = cscale(Dk[e], s);
  }
  __syncthreads();
  double cost = 0.0;
  double2* E = cta_expm(X, Y2, Y3, Y4, R, T, W, red, &cost);
  if (threadIdx.x == 0) atomicAdd(&st->exp_products, cost + 1.0);
  // E is R or T; reuse X/Y2 for U
  double2* dUk = P.dU + (size_t)k * WW;
  const int cur = st->cur;
  const double2* Uk = P.U[cur] + (size_t)k * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    dUk[e] = E[e];
    X[e] = Uk[e];
  }
  __syncthreads();
  cta_gemm<false>(Y2, W, X, W, E, W, W);
  __syncthreads();
  double2* Un = P.U[cur ^ 1] + (size_t)k * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) Un[e] = Y2[e];
}

// ----------------------------------------------------------------------------
// k_m_update: M(k,b) <- dU(k)^H M(k,b) dU(nnlist(k,b))   (src/wannierise.F90:1736-1748)
// mode 0: step update, reads M[cur], writes M[cur^1] (which selects trial/optimal pass)
// mode 1: projection (src/overlap.F90:909-923): rotation U[cur], in place on M[cur].
// Epilogue: block statistics for the spread passes.  One CTA (256 threads) per (problem, k*B+b).
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_m_update(const Problem* __restrict__ probs, WorkMap wm,
                                                  int mode, int which) {
  extern __shared__ double2 smem[];
  __shared__ double red[256];
  int kb;
  const int p = locate(wm, blockIdx.x, kb);
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (mode == 0) {
    if (st->done) return;
    if (which == 1 && !st->do_second) return;
  }
  const int W = P.W, WW = W * W, B = P.B;
  const int k = kb / B;
  const int k2 = P.nnlist[kb];
  const int cur = st->cur;
  const double2* rot = (mode == 0) ? P.dU : P.U[cur];
  const double2* Rk = rot + (size_t)k * WW;
  const double2* Rk2 = rot + (size_t)k2 * WW;
  const double2* Min = P.M[cur] + (size_t)kb * WW;
  double2* Mout = P.M[mode == 0 ? (cur ^ 1) : cur] + (size_t)kb * WW;
  if (W <= kSmemW) {
    double2 *sR = smem, *sM = smem + WW, *sR2 = smem + 2 * WW, *sT = smem + 3 * WW;
    for (int e = threadIdx.x; e < WW; e += blockDim.x) {
      sR[e] = Rk[e];
      sM[e] = Min[e];
      sR2[e] = Rk2[e];
    }
    __syncthreads();
    cta_gemm<true>(sT, W, sR, W, sM, W, W);
    __syncthreads();
    cta_gemm<false>(sM, W, sT, W, sR2, W, W);
    __syncthreads();
    for (int e = threadIdx.x; e < WW; e += blockDim.x) Mout[e] = sM[e];
    block_stats(sM, W, W, P.diag_ln + (size_t)kb * W, P.diag_abs2 + (size_t)kb * W, P.offd + kb, red, &P,
                (size_t)kb);
  } else {
    // operands stay in global memory (L1/L2-resident); T = R(k)^H M(k,b) in tbuf
    double2* Tg = P.tbuf + (size_t)kb * WW;
    cta_gemm<true>(Tg, W, Rk, W, Min, W, W);
    __syncthreads();
    cta_gemm<false>(Mout, W, Tg, W, Rk2, W, W);
    __syncthreads();
    block_stats(Mout, W, W, P.diag_ln + (size_t)kb * W, P.diag_abs2 + (size_t)kb * W, P.offd + kb, red, &P,
                (size_t)kb);
  }
}

// ----------------------------------------------------------------------------
// k_ctrl_step: internal_optimal_step (src/wannierise.F90:1528-1596).  One thread per problem.
// ----------------------------------------------------------------------------
__global__ void k_ctrl_step(const Problem* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (st->done) return;
  const Control& c = P.ctl;
  if (c.lfixstep) {
    st->lquad = 0;
    st->do_second = 0;
    return;
  }
  const double trial = st->slot[0].om_tot, cur = st->wann.om_tot;
  double fac = trial - cur, shift;
  if (fabs(fac) > 2.2250738585072014e-308) {   // tiny(1.0_dp)
    fac = 1.0 / fac;
    shift = 1.0;
  } else {
    fac = 1.0e6;
    shift = fac * trial - fac * cur;
  }
  const double eqb = fac * st->doda0;
  const double eqa = shift - eqb * c.trial_step;
  int lquad;
  double alphamin, falphamin;
  if (fabs(eqa / (fac * cur)) > 2.220446049250313e-16) {
    lquad = 1;
    alphamin = -0.5 * eqb / eqa * (c.trial_step * c.trial_step);
    falphamin = cur - 0.25 * eqb * eqb / (fac * eqa) * (c.trial_step * c.trial_step);
  } else {
    lquad = 0;
    alphamin = c.trial_step;
    falphamin = trial;
  }
  if (st->doda0 * alphamin > 0.0) {
    lquad = 0;
    alphamin = c.trial_step;
    falphamin = trial;
  }
  st->lquad = lquad;
  st->alphamin = alphamin;
  st->falphamin = falphamin;
  st->do_second = lquad;
  st->s_second = alphamin / (4.0 * P.wbtot);
}

// ----------------------------------------------------------------------------
// k_ctrl_end: spread bookkeeping, log line, convergence (internal_test_convergence,
// src/wannierise.F90:1076-1164), buffer flip.  One CTA (128 threads) per problem.
// ----------------------------------------------------------------------------
__global__ void k_ctrl_end(const Problem* __restrict__ probs) {
  const Problem& P = probs[blockIdx.x];
  CtrlState* st = P.st;
  if (st->done) return;
  const int W = P.W;
  const int acc = st->do_second ? 1 : 0;
  // accepted centres -> slot 2
  const double* src = P.centres + (size_t)acc * 4 * W;
  double* dst = P.centres + (size_t)2 * 4 * W;
  double* lgc = P.log_centres + (size_t)(st->iter + 1) * 4 * W;
  for (int i = threadIdx.x; i < 4 * W; i += blockDim.x) {
    dst[i] = src[i];
    lgc[i] = src[i];
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const Control& c = P.ctl;
  st->old = st->wann;
  st->wann = st->slot[acc];
  st->cur ^= 1;
  const int iter = st->iter + 1;
  st->iter = iter;
  double* lg = P.log + (size_t)iter * kLogStride;
  lg[0] = iter;
  lg[1] = st->wann.om_tot - st->old.om_tot;
  lg[2] = sqrt(fabs(st->gcnorm1));
  lg[3] = st->wann.om_tot;
  lg[4] = st->wann.om_d;
  lg[5] = st->wann.om_od;
  lg[6] = st->lquad;
  lg[7] = st->alphamin;
  unsigned long long tns;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tns));
  lg[8] = (double)tns;
  lg[9] = st->wann.om_nu;
  if (c.conv_window > 1) {
    const double delta = st->wann.om_tot - st->old.om_tot;
    const int cw = c.conv_window;
    if (iter <= cw) {
      st->history[iter - 1] = delta;
    } else {
      for (int j = 0; j < cw - 1; ++j) st->history[j] = st->history[j + 1];
      st->history[cw - 1] = delta;
    }
    st->conv_count += 1;
    if (st->conv_count >= cw) {
      bool ok = true;
      for (int j = 0; j < cw; ++j)
        if (fabs(st->history[j]) > c.conv_tol) ok = false;
      if (ok) st->lconverged = 1;   // conv_noise_amp > 0 is rejected on the host
    }
  }
  if (st->lconverged || iter >= c.num_iter) st->done = 1;
  if (!isfinite(st->wann.om_tot)) {
    st->error = 1;
    st->done = 1;
  }
}

// ----------------------------------------------------------------------------
// k_log_init: log row 0 = the "Initial State" block (src/wannierise.F90:479-520).
// ----------------------------------------------------------------------------
__global__ void k_log_init(const Problem* __restrict__ probs) {
  const Problem& P = probs[blockIdx.x];
  const int W = P.W;
  const double* src = P.centres + (size_t)2 * 4 * W;
  for (int i = threadIdx.x; i < 4 * W; i += blockDim.x) P.log_centres[i] = src[i];
  if (threadIdx.x == 0) {
    CtrlState* st = P.st;
    if (P.guiding && P.no_guide_iter <= 0) st->irguide = 1;   // src/wannierise.F90:435-443
    double* lg = P.log;
    lg[0] = 0;
    lg[1] = st->wann.om_tot;
    lg[2] = 0.0;
    lg[3] = st->wann.om_tot;
    lg[4] = st->wann.om_d;
    lg[5] = st->wann.om_od;
    lg[6] = 0;
    lg[7] = 0;
    unsigned long long tns;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tns));
    lg[8] = (double)tns;
    lg[9] = st->wann.om_nu;
  }
}

// ----------------------------------------------------------------------------
// k_lowdin: overlap_project's U(k) = Z V^dagger from A(k) = Z S V^dagger
// (src/overlap.F90:842-860), computed as U = A (A^H A)^{-1/2} = A V L^{-1/2} V^H with the
// Jacobi eigenpairs (V, L) of A^H A: the same unitary polar factor for full-rank A.
// Input A(k) in U[cur](k) (the reference reads A into u_matrix, src/wannier_prog.F90:523-529);
// output U overwrites it.  One CTA (256 threads) per (problem, k).
// Status per k: 0 ok, 1 rank deficient, 2 Jacobi not converged.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_lowdin(const Problem* __restrict__ probs, WorkMap wm,
                                                int* __restrict__ status) {
  extern __shared__ double2 smem[];
  __shared__ double red[256];
  __shared__ double rc[128];
  __shared__ double2 rse[128];
  __shared__ int rp[128], rq[128];
  int k;
  const int p = locate(wm, blockIdx.x, k);
  const Problem& P = probs[p];
  const int W = P.W, WW = W * W;
  double2* buf = (W <= kSmemW) ? smem : (P.work + (size_t)k * 6 * WW);
  double2 *A = buf, *S = buf + WW, *V = buf + 2 * WW, *T = buf + 3 * WW;
  double2* Uk = P.U[P.st->cur] + (size_t)k * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) A[e] = Uk[e];
  __syncthreads();
  cta_gemm<true>(S, W, A, W, A, W, W);
  __syncthreads();
  const int sweeps = cta_jacobi(S, V, W, 60, red, rc, rse, rp, rq);
  // V' = V diag(lambda^{-1/2}) into T
  __shared__ int bad;
  if (threadIdx.x == 0) bad = (sweeps < 0) ? 2 : 0;
  __syncthreads();
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    const int j = e / W;
    const double l = S[j * W + j].x;
    if (!(l > 0.0)) bad = 1;
    T[e] = cscale(V[e], 1.0 / sqrt(l));
  }
  __syncthreads();
  cta_gemm<false>(S, W, A, W, T, W, W);      // S <- A V L^{-1/2}
  __syncthreads();
  // U = S V^H : compute via (V S^H)^H  -> use conj-transposed product with A := V
  // U_ij = sum_l S_il conj(V_jl)
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    const int i = e % W, j = e / W;
    double2 acc = cmk(0, 0);
    for (int l = 0; l < W; ++l) {
      const double2 s = S[l * W + i];
      const double2 v = V[l * W + j];
      acc = cadd(acc, cmulc(s, v));
    }
    Uk[e] = acc;
  }
  if (threadIdx.x == 0) status[blockIdx.x] = bad;
}

// ----------------------------------------------------------------------------
// k_unitarity: wann_check_unitarity (src/wannierise.F90:2594-2661); writes
// max(|U U^H - I|, |U^H U - I|) per (problem, k).  One CTA (128 threads) per item.
// ----------------------------------------------------------------------------
__global__ void k_unitarity(const Problem* __restrict__ probs, WorkMap wm, double* __restrict__ out) {
  __shared__ double red[128];
  int k;
  const int p = locate(wm, blockIdx.x, k);
  const Problem& P = probs[p];
  const int W = P.W;
  const double2* U = P.U[P.st->cur] + (size_t)k * W * W;
  double mx = 0.0;
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
    const int i = e % W, j = e / W;
    double2 a = cmk(0, 0), b = cmk(0, 0);
    for (int m = 0; m < W; ++m) {
      a = cadd(a, cmulc(U[m * W + i], U[m * W + j]));      // (U U^H)_ij
      b = cadd(b, cmulc(U[j * W + m], U[i * W + m]));      // (U^H U)_ij
    }
    if (i == j) {
      a.x -= 1.0;
      b.x -= 1.0;
    }
    mx = fmax(mx, fmax(sqrt(cabs2(a)), sqrt(cabs2(b))));
  }
  mx = block_max(mx, red);
  if (threadIdx.x == 0) out[blockIdx.x] = mx;
}

// ----------------------------------------------------------------------------
// k_all_done: *out = 1 when every problem of the batch has finished.
// ----------------------------------------------------------------------------
__global__ void k_all_done(const Problem* __restrict__ probs, int nprob, int* __restrict__ out) {
  __shared__ int active;
  if (threadIdx.x == 0) active = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < nprob; p += blockDim.x)
    if (!probs[p].st->done) active = 1;
  __syncthreads();
  if (threadIdx.x == 0) *out = active ? 0 : 1;
}

// ----------------------------------------------------------------------------
// k_fp64_peak: FP64 FMA throughput probe (8 independent dependency chains per thread).
// Used to state the FP64-pipe roofline, which the measured-peaks file does not carry.
// ----------------------------------------------------------------------------
__global__ void k_fp64_peak(double* __restrict__ out, int iters, double seed) {
  double a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + threadIdx.x * 1e-9 + i;
  const double m = 0.999999999, c = 1e-12;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma(a[i], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == 12345.678) out[0] = s;   // keeps the chains live; never true for these inputs
}

// ----------------------------------------------------------------------------
// Tensor-path bookkeeping: during the loop U[] holds R = U0^H U (identity at entry),
// M is always recomputed from the entry overlaps M0; at the end U = U0 R.
// k_u_identity: U[0](k) = I.   k_u_final: U[cur](k) <- U0(k) U[cur](k).
// One CTA (256 threads) per (problem, k).
// ----------------------------------------------------------------------------
__global__ void k_u_identity(const Problem* __restrict__ probs, WorkMap wm) {
  int k;
  const int p = locate(wm, blockIdx.x, k);
  const Problem& P = probs[p];
  const int W = P.W;
  double2* U = P.U[0] + (size_t)k * W * W;
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) U[e] = cmk((e % W) == (e / W) ? 1.0 : 0.0, 0.0);
}

__global__ void __launch_bounds__(256) k_u_final(const Problem* __restrict__ probs, WorkMap wm) {
  extern __shared__ double2 smem[];
  int k;
  const int p = locate(wm, blockIdx.x, k);
  const Problem& P = probs[p];
  const int W = P.W, WW = W * W;
  double2* R = P.U[P.st->cur] + (size_t)k * WW;
  const double2* U0 = P.U0 + (size_t)k * WW;
  double2* buf = (W <= kSmemW) ? smem : (P.work + (size_t)k * 6 * WW);
  double2 *sA = buf, *sR = buf + WW, *sC = buf + 2 * WW;
  for (int e = threadIdx.x; e < WW; e += blockDim.x) {
    sA[e] = U0[e];
    sR[e] = R[e];
  }
  __syncthreads();
  cta_gemm<false>(sC, W, sA, W, sR, W, W);
  __syncthreads();
  for (int e = threadIdx.x; e < WW; e += blockDim.x) R[e] = sC[e];
}

// ----------------------------------------------------------------------------
// k_frob0: |M0(k,b)|_F^2 per block (tensor path, once per solve).  One CTA per (k,b).
// ----------------------------------------------------------------------------
__global__ void k_frob0(const Problem* __restrict__ probs, WorkMap wm) {
  __shared__ double red[128];
  int kb;
  const int p = locate(wm, blockIdx.x, kb);
  const Problem& P = probs[p];
  const int W = P.W;
  const double2* Mb = P.M0 + (size_t)kb * W * W;
  double acc = 0.0;
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) acc += cabs2(Mb[e]);
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) P.frob0[kb] = acc;
}

}  // namespace w90g
