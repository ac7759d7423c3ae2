// Tensor-core M update: M(k,b) = U(k)^H M0(k,b) U(k+b) with FP64-level accuracy from
// FP16 tcgen05 MMAs (Ozaki-style exact slicing).
//
// Every complex product is computed through its real embedding
//     [C_r C_i] = [A_r A_i] [[B_r, B_i], [-B_i, B_r]]      (K = N = 2*WP real)
// Each operand is scaled per row (A) / per column (B) by a power of two and split into
// S = 7 signed 7-bit digits (x_1 in [-128,128], x_t in [-64,63] for t > 1), each an exact
// FP16 value (built two at a time by a packed FP16 subtraction, pack_digits7).  For every digit pair (t,u) with t+u <= S-1 (0-based) the MMA A^(t) B^(u)
// over the K = 2*WP reduction is exact in the FP32 accumulator (every partial sum is an
// integer below 2^22), so the pairs of one diagonal d = t+u share one TMEM accumulator.
// The epilogue recombines the 7 diagonals exactly in int64 and rounds once to FP64.
// Truncation error: ~2^-49 relative to (row scale x column scale) per product term.
// Widths up to 128 are handled by chunking K and N in 32-complex-column pieces.
//
// The product is batched as tall-skinny GEMMs (B*WP rows sharing one WP x WP operand):
//   step 1 (group k):  rows (b, n):  Z(k,b)^T = M0(k,b)^T conj(U(k))   -> Z row-major
//   step 2 (group k'): rows of Z(k,b) for the B pairs with nnlist(k,b) = k':
//                      M(k,b) = Z(k,b) U(k')  -> M column-major + block statistics
// One CTA per group; 128-row tiles; operands sliced by all 256 threads into shared
// memory (canonical K-major, no swizzle); one thread issues the MMAs; warps 0-3 read
// the accumulators (TMEM lanes = rows).
#include "oz.cuh"

namespace w90g {

// Digit scheme: 7 signed 7-bit digits (49 bits).  (8-bit digits give 56 bits for the
// same 28 MMAs but their wider exact recombination made the update 20% slower; the
// update's ~2^-49 error stays far below what the line search resolves.)
template <int WP>
__device__ __forceinline__ void split_digits(double v, int e, int x[kS]) {
  digits7(scaled_int(v, e), x);
}

// value of the 7 FP32 diagonal accumulators dd[0], dd[stride], ... for row / column
// exponents summing to escale
template <int WP>
__device__ __forceinline__ double recombine_digits(const uint32_t* dd, int stride, int escale) {
  long long acc = float_to_int_exact(__uint_as_float(dd[0]));
#pragma unroll
  for (int d = 1; d < kDiag; ++d) acc = (acc << 7) + float_to_int_exact(__uint_as_float(dd[d * stride]));
  return int64_scaled_to_double(acc, escale - 56);
}

// Row exponents of A tile `tile` (2 threads per row, all 256 threads of the CTA).
template <int WP, class AElem>
__device__ __forceinline__ void a_row_exponents(int tile, int W, int* rowexp, AElem&& a_elem) {
  const int tid = threadIdx.x;
  const int r = tid >> 1, half = tid & 1;
  const int row = tile * kTileRows + r;
  unsigned long long mx = 0ull;
  // eight independent loads in flight per round (the max does not depend on the order)
  for (int m0 = half; m0 < W; m0 += 16) {
    double2 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (m0 + 2 * i < W) ? a_elem(row, m0 + 2 * i) : make_double2(0.0, 0.0);
#pragma unroll
    for (int i = 0; i < 8; ++i) mx = max(mx, max(abs_bits(v[i].x), abs_bits(v[i].y)));
  }
  mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mx, 1));
  if (half == 0) rowexp[r] = exp_above_bits(mx);
}

// The kS digit planes of A chunk (tile, kc) in the canonical K-major layout, written to
// dst (shared memory, or the global image the shared-memory copy is taken from).  A
// thread slices one part (re / im) of 8 consecutive K of one row -- one 16-byte core row
// per plane -- and lanes take consecutive rows, so the 16-byte stores do not conflict.
template <int WP, class AElem>
__device__ __forceinline__ void a_slice_chunk(unsigned char* dst, int tile, int kc, const int* rowexp,
                                              AElem&& a_elem) {
  using L = TileSmem<WP>;
  constexpr int CW = L::CW, KC = L::KC, LG = CW / 8;
  for (int it = threadIdx.x; it < kTileRows * LG * 2; it += blockDim.x) {
    const int r = it % kTileRows, lg = (it / kTileRows) % LG, part = it / (kTileRows * LG);
    double v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const double2 a = a_elem(tile * kTileRows + r, kc * CW + lg * 8 + i);
      v[i] = part == 0 ? a.x : a.y;
    }
    uint32_t w[kS][4];
    pack_digits7(w, v, rowexp[r], false);
    const uint32_t o = kmaj_off(r, part * CW + lg * 8, KC);
#pragma unroll
    for (int t = 0; t < kS; ++t)
      *(uint4*)(dst + (size_t)t * L::A_BYTES + o) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
  }
}

// STEP 1: group = k.  STEP 2: group = k'.  which: 0 trial, 1 optimal-step pass.
template <int WP, int STEP>
__global__ void __launch_bounds__(256, 1) k_oz_mupdate(const Problem* __restrict__ probs, WorkMap wm, int which) {
  using L = TileSmem<WP>;
  constexpr int CW = L::CW, KC = L::KC, NC = L::NC, NCH = L::NCH;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;                                   // kS slices of an A chunk
  unsigned char* sB = base + (size_t)kS * L::A_BYTES;          // kS slices of a B chunk
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t mbar_ld;   // completion of the bulk copies of presliced A
  __shared__ uint32_t tmem_base_slot;
  __shared__ int s_rowexp[kTileRows];
  __shared__ int s_colexp[WP];
  __shared__ int s_bad;

  int g;
  const int p = locate(wm, blockIdx.x, g);
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (st->done) return;
  if (which == 1 && !st->do_second) return;
  const int W = P.W, B = P.B, WW = W * W;
  const int cur = st->cur;
  const double2* Unew = P.U[cur ^ 1];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // ---- TMEM allocation (warp 0) and barrier init
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(&tmem_base_slot)), "r"((uint32_t)L::TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar_ld)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_bad = 0;
  }

  // ---- B operand of the group: step 1 conj(U(k)), step 2 U(k'); B(K=m, N=c) = (conj) U(m, c)
  const double2* Ug = Unew + (size_t)g * WW;
  {
    // column scales: 256 / WP threads per column, four independent loads per round, a max
    // across those lanes
    constexpr int TPC = 256 / WP;
    const int c = tid / TPC, sub = tid % TPC;
    unsigned long long mx = 0ull;
    if (c < W)
      for (int m0 = sub; m0 < W; m0 += 4 * TPC) {
        double2 v[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int m = m0 + i * TPC;
          v[i] = (m < W) ? Ug[(size_t)c * W + m] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) mx = max(mx, max(abs_bits(v[i].x), abs_bits(v[i].y)));
      }
#pragma unroll
    for (int o = 1; o < TPC; o <<= 1)
      mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mx, o));
    if (sub == 0 && c < WP) s_colexp[c] = exp_above_bits(mx);
  }

  // slice the (nc, kc) chunk of B^T (K-major: rows = real N index within the chunk): a
  // thread takes 8 consecutive K of one row n, i.e. one entry of the embedding
  // [[B_r, B_i], [-B_i, B_r]] for 8 consecutive m of column c (contiguous in memory), and
  // writes one 16-byte core row per plane
  auto slice_b = [&](int nc, int kc) {
    constexpr int KG = KC / 8;
    for (int it = tid; it < NC * KG; it += blockDim.x) {
      const int n = it % NC, kk0 = (it / NC) * 8;
      const bool nre = n < CW, kre = kk0 < CW;
      const int cc = nc * CW + (nre ? n : n - CW);      // complex column
      const int mm0 = kc * CW + (kre ? kk0 : kk0 - CW); // complex row (K index) of the first
      double v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int mm = mm0 + i;
        v[i] = 0.0;
        if (cc < W && mm < W) {
          const double2 u = Ug[(size_t)cc * W + mm];
          const double br = u.x, bi = (STEP == 1) ? -u.y : u.y;
          v[i] = (kre && nre) ? br : (kre ? bi : (nre ? -bi : br));   // [B_r B_i; -B_i B_r]
        }
      }
      uint32_t w[kS][4];
      pack_digits7(w, v, s_colexp[cc < WP ? cc : 0], false);
      const uint32_t off = kmaj_off(n, kk0, KC);
#pragma unroll
      for (int t = 0; t < kS; ++t)
        *(uint4*)(sB + (size_t)t * L::B_BYTES + off) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
    }
  };

  const int rows_group = B * WP;
  const int ntiles = (rows_group + kTileRows - 1) / kTileRows;
  __syncthreads();
  if (NCH == 1) slice_b(0, 0);
  const uint32_t tmem = tmem_base_slot;
  uint32_t phase = 0, phase_ld = 0;

  // A element (row, complex K index m) of this tile
  auto a_elem = [&](int row, int m) -> double2 {
    const int bi = row / WP, rr = row % WP;
    if (bi >= B || rr >= W || m >= W) return make_double2(0.0, 0.0);
    if (STEP == 1) return P.M0[((size_t)g * B + bi) * WW + (size_t)rr * W + m];   // M0(k,b)(m, n=rr)
    const int kb = P.inv_nnlist[(size_t)g * B + bi];
    return P.tbuf[(size_t)kb * WW + (size_t)rr * W + m];                          // Z(k,b)(m=rr, j=m), row-major
  };

  // step 1 takes its A operand (the entry overlaps, fixed for the whole solve) from the
  // digit planes sliced once by k_oz_preslice: the same bytes, copied instead of computed
  const bool presliced = (STEP == 1) && (P.m0s != nullptr);
  for (int tile = 0; tile < ntiles; ++tile) {
    // ---- row scales over the full row (2 threads per row)
    if (presliced) {
      if (tid < kTileRows) s_rowexp[tid] = P.m0s_exp[((size_t)g * ntiles + tile) * kTileRows + tid];
    } else {
      a_row_exponents<WP>(tile, W, s_rowexp, a_elem);
    }
    __syncthreads();
    for (int nc = 0; nc < NCH; ++nc) {
      bool ok = true;
      for (int kc = 0; kc < NCH; ++kc) {
        // ---- the kc chunk of A: kS digit planes, either copied by the bulk-copy engine
        // from the presliced image (one cp.async.bulk per plane, completion counted in bytes
        // on mbar_ld; sA is free: the previous MMAs completed before their epilogue) or
        // sliced here
        if (presliced) {
          if (tid == 0) {
            const unsigned char* src = P.m0s + (((size_t)g * ntiles + tile) * NCH + kc) * (size_t)kS * L::A_BYTES;
            asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                         :: "r"(smem_u32(&mbar_ld)), "r"((uint32_t)(kS * L::A_BYTES)) : "memory");
#pragma unroll
            for (int t = 0; t < kS; ++t)
              asm volatile(
                  "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                  :: "r"(smem_u32(sA + (size_t)t * L::A_BYTES)), "l"(src + (size_t)t * L::A_BYTES),
                     "r"((uint32_t)L::A_BYTES), "r"(smem_u32(&mbar_ld))
                  : "memory");
          }
        } else {
          a_slice_chunk<WP>(sA, tile, kc, s_rowexp, a_elem);
        }
        if (NCH > 1) slice_b(nc, kc);
        if (presliced) {
          // bounded wait, by the MMA-issuing thread alone (the only reader of the copied
          // planes); on a timeout the error is recorded and the drain wait lets the copies
          // in flight land before the CTA gives up its shared memory
          if (tid == 0 && !mbar_wait(smem_u32(&mbar_ld), phase_ld)) {
            s_bad = 1;
            mbar_drain(smem_u32(&mbar_ld), phase_ld);
          }
          phase_ld ^= 1u;
        }
        // generic-proxy smem writes -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (s_bad) {
          ok = false;
          break;
        }
        // ---- MMAs: digit pairs (t,u), t+u <= S-1 (0-based) -> accumulator of diagonal t+u
        if (tid == 0) {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // descriptors: the base descriptor plus the byte offset / 16 in the address field
          // (shared-memory addresses stay below 2^18, so the field holds it)
          const uint64_t da = smem_desc(smem_u32(sA), 128, (KC / 8) * 128);
          const uint64_t db = smem_desc(smem_u32(sB), 128, (KC / 8) * 128);
          // B's digit planes follow one another as row groups of one K-major operand and
          // diagonal d's accumulator columns follow d - 1's: slice t of A against planes
          // u0 .. u0 + n - 1 of B is one MMA with N = n NC (<= 256), writing diagonals t + u0 ..
          constexpr int PPM = 256 / NC;
#pragma unroll
          for (int t = 0; t < kS; ++t) {
#pragma unroll
            for (int u0 = 0; u0 + t <= kS - 1; u0 += PPM) {
              const int n = (kS - t - u0) < PPM ? (kS - t - u0) : PPM;
              const uint32_t dtm = tmem + (uint32_t)((t + u0) * NC);
              // the first write of every diagonal in this N chunk: slice 0 of A, chunk kc = 0
              const bool first_pair = (kc == 0) && (t == 0);
#pragma unroll
              for (int ks = 0; ks < KC / 16; ++ks) {
                const uint64_t ad = da + (uint64_t)(((size_t)t * L::A_BYTES + ks * 256) >> 4);
                const uint64_t bd = db + (uint64_t)(((size_t)u0 * L::B_BYTES + ks * 256) >> 4);
                const uint32_t acc = (first_pair && ks == 0) ? 0u : 1u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    :: "r"(dtm), "l"(ad), "l"(bd), "r"(idesc_f16(n * NC)), "r"(acc)
                    : "memory");
              }
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                       :: "r"(smem_u32(&mbar)) : "memory");
        }
        // one thread waits for the commit (the others wait at the CTA barrier below)
        const bool ok_mine = (tid != 0) || mbar_wait(smem_u32(&mbar), phase);
        if (!ok_mine) {
          // the MMAs may still run: record the error, then wait (drain limit) for their
          // commit before the CTA reads or frees tensor memory or reuses the operands
          s_bad = 1;
          mbar_drain(smem_u32(&mbar), phase);
        }
        phase ^= 1u;
        __syncthreads();
        ok = (s_bad == 0);   // uniform across the CTA
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!ok) break;
      }
      // ---- epilogue for N chunk nc: all 8 warps; warp w reads TMEM lanes 32*(w%4)..,
      // warps w and w+4 take the lower / upper half of the chunk's CW complex columns
      if (ok) {
        const int wq = warp & 3, half = warp >> 2;
        const int r = wq * 32 + lane;
        const int row = tile * kTileRows + r;
        const int bi = row / WP, rr = row % WP;
        const bool valid = (bi < B) && (rr < W);
        const int erow = s_rowexp[r];
        const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
        int kb_out = 0;
        if (STEP == 2 && bi < B) kb_out = P.inv_nnlist[(size_t)g * B + bi];
        const int jbeg = half * (CW / 2), jend = jbeg + CW / 2;
        double dre = 0.0, dim = 0.0;
        bool has_diag = false;
#pragma unroll 1
        for (int j0 = jbeg; j0 < jend; j0 += 4) {
          uint32_t q[kDiag][4], s4[kDiag][4];
#pragma unroll
          for (int d = 0; d < kDiag; ++d) {
            const uint32_t ta = tmem + lane_base + (uint32_t)(d * NC + j0);
            const uint32_t tb = tmem + lane_base + (uint32_t)(d * NC + CW + j0);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(q[d][0]), "=r"(q[d][1]), "=r"(q[d][2]), "=r"(q[d][3])
                         : "r"(ta));
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(s4[d][0]), "=r"(s4[d][1]), "=r"(s4[d][2]), "=r"(s4[d][3])
                         : "r"(tb));
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int c = nc * CW + j0 + j;   // complex output column
            // S = sum_d D_d 2^(7(6-d)) by Horner in int64 (exact, |S| < 2^63)
            const int ecol = s_colexp[c < WP ? c : 0];
            const double re = recombine_digits<WP>(&q[0][j], 4, erow + ecol);
            const double im = recombine_digits<WP>(&s4[0][j], 4, erow + ecol);
            if (valid && c < W) {
              if (STEP == 1) {
                // Z(k,b) row-major: element (j=c, n=rr) at c*W + rr
                P.tbuf[((size_t)g * B + bi) * WW + (size_t)c * W + rr] = make_double2(re, im);
              } else {
                // M(k,b) column-major: element (m=rr, c) at c*W + rr
                P.M[cur ^ 1][(size_t)kb_out * WW + (size_t)c * W + rr] = make_double2(re, im);
                if (c == rr) {
                  dre = re;
                  dim = im;
                  has_diag = true;
                }
              }
            }
          }
        }
        if (STEP == 2 && has_diag) {
          // diagonal statistics (once per row); the off-diagonal sum follows from the
          // invariant |M(k,b)|_F^2 = |M0(k,b)|_F^2 in the spread pass
          P.diag_ln[(size_t)kb_out * W + rr] = guided_ln(P, (size_t)kb_out * W + rr, make_double2(dre, dim));
          P.diag_abs2[(size_t)kb_out * W + rr] = dre * dre + dim * dim;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (s_bad) break;
    }
    if (s_bad) break;
  }
  if (s_bad && tid == 0) {
    st->error = 2;
    st->done = 1;
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(tmem), "r"((uint32_t)L::TMEM_COLS) : "memory");
  }
}

// Slices step 1's A operand once per solve: for every k, tile and K chunk, the kS digit
// planes exactly as k_oz_mupdate<WP, 1> would write them to shared memory, plus the tile's
// row exponents.  One CTA (256 threads) per k.
template <int WP>
__global__ void __launch_bounds__(256) k_oz_preslice(const Problem* __restrict__ probs, WorkMap wm) {
  using L = TileSmem<WP>;
  constexpr int NCH = L::NCH;
  __shared__ int s_rowexp[kTileRows];
  int g;
  const int p = locate(wm, blockIdx.x, g);
  const Problem& P = probs[p];
  if (!P.m0s) return;
  const int W = P.W, B = P.B, WW = W * W;
  const int ntiles = (B * WP + kTileRows - 1) / kTileRows;
  auto a_elem = [&](int row, int m) -> double2 {
    const int bi = row / WP, rr = row % WP;
    if (bi >= B || rr >= W || m >= W) return make_double2(0.0, 0.0);
    return P.M0[((size_t)g * B + bi) * WW + (size_t)rr * W + m];
  };
  for (int tile = 0; tile < ntiles; ++tile) {
    a_row_exponents<WP>(tile, W, s_rowexp, a_elem);
    __syncthreads();
    if (threadIdx.x < kTileRows) P.m0s_exp[((size_t)g * ntiles + tile) * kTileRows + threadIdx.x] = s_rowexp[threadIdx.x];
    for (int kc = 0; kc < NCH; ++kc)
      a_slice_chunk<WP>(P.m0s + (((size_t)g * ntiles + tile) * NCH + kc) * (size_t)kS * L::A_BYTES, tile, kc,
                        s_rowexp, a_elem);
    __syncthreads();
  }
}

// bytes of the pre-sliced A operand and of its row exponents for K k-points, B neighbours
void oz_preslice_bytes(int wp, int K, int B, size_t* data, size_t* exps) {
  const int cw = wp < 32 ? wp : 32;
  const size_t a_bytes = (size_t)kTileRows * 2 * cw * 2;
  const size_t ntiles = ((size_t)B * wp + kTileRows - 1) / kTileRows;
  *data = (size_t)K * ntiles * (wp / cw) * kS * a_bytes;
  *exps = (size_t)K * ntiles * kTileRows * 4;
}

cudaError_t oz_preslice_launch(int wp, const Problem* probs, WorkMap wm, int grid, cudaStream_t s) {
  switch (wp) {
    case 8: k_oz_preslice<8><<<grid, 256, 0, s>>>(probs, wm); break;
    case 16: k_oz_preslice<16><<<grid, 256, 0, s>>>(probs, wm); break;
    case 32: k_oz_preslice<32><<<grid, 256, 0, s>>>(probs, wm); break;
    case 64: k_oz_preslice<64><<<grid, 256, 0, s>>>(probs, wm); break;
    case 128: k_oz_preslice<128><<<grid, 256, 0, s>>>(probs, wm); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// host-side launchers (the template kernels stay private to this translation unit)
template <int WP>
static cudaError_t oz_launch_wp(int step, const Problem* probs, WorkMap wm, int which, int grid,
                                cudaStream_t s) {
  const size_t sm = TileSmem<WP>::BYTES;
  if (step == 1) k_oz_mupdate<WP, 1><<<grid, 256, sm, s>>>(probs, wm, which);
  else k_oz_mupdate<WP, 2><<<grid, 256, sm, s>>>(probs, wm, which);
  return cudaGetLastError();
}

cudaError_t oz_launch(int wp, int step, const Problem* probs, WorkMap wm, int which, int grid,
                      cudaStream_t s) {
  switch (wp) {
    case 8: return oz_launch_wp<8>(step, probs, wm, which, grid, s);
    case 16: return oz_launch_wp<16>(step, probs, wm, which, grid, s);
    case 32: return oz_launch_wp<32>(step, probs, wm, which, grid, s);
    case 64: return oz_launch_wp<64>(step, probs, wm, which, grid, s);
    default: return oz_launch_wp<128>(step, probs, wm, which, grid, s);
  }
}

template <int WP>
static cudaError_t oz_attr_wp() {
  const int sm = (int)TileSmem<WP>::BYTES;
  cudaError_t e = cudaFuncSetAttribute(k_oz_mupdate<WP, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_oz_mupdate<WP, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
}

cudaError_t oz_set_attributes(int wp) {
  switch (wp) {
    case 8: return oz_attr_wp<8>();
    case 16: return oz_attr_wp<16>();
    case 32: return oz_attr_wp<32>();
    case 64: return oz_attr_wp<64>();
    default: return oz_attr_wp<128>();
  }
}

size_t oz_smem_bytes(int wp) {
  switch (wp) {
    case 8: return TileSmem<8>::BYTES;
    case 16: return TileSmem<16>::BYTES;
    case 32: return TileSmem<32>::BYTES;
    case 64: return TileSmem<64>::BYTES;
    default: return TileSmem<128>::BYTES;
  }
}

}  // namespace w90g
