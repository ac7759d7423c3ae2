// Tensor-core rotation step: dU(k) = exp(s D(k)) and U(k) <- U(k) dU(k)
// (internal_new_u_and_m, src/wannierise.F90:1655-1733) with every W x W complex
// product on the tcgen05 tensor cores through exact slicing into BF16 / FP16 digits
// (see k_tensor.cu).
//
// The matrix function is the FP64 path's (k_exp_u in k_fp64.cu): scaling and squaring
// of a Taylor polynomial evaluated by Paterson-Stockmeyer, degree and squarings chosen
// per matrix from its 1-norm.  Scalar work (norms, the polynomial's linear combinations,
// the Hermitian symmetrisation of the even powers) stays in FP64; only the products move
// to the tensor pipe.  The exp chain (powers, Horner steps, up to ~10 squarings that
// double any error) needs 56-bit operands: a product is accurate to ~2^-56 of
// (row scale x column scale), below FP64 GEMM roundoff.  Two product forms:
//   num_wann <= 64: [C_r; C_i] = [[A_r, -A_i], [A_i, A_r]] [B_r; B_i], 7 signed 8-bit
//     digits (FP16 operands), 28 digit pairs (oz_cmm2);
//   num_wann = 65..128: [C_r C_i] = [A_r A_i] [[B_r, B_i], [-B_i, B_r]], 8 signed
//     7-bit digits, 36 digit pairs (oz_cmm; K = 256 keeps 8-bit digits from being exact).
//
// One CTA (256 threads) per (problem, k).  A product puts the rows of its A operand on
// the 128 TMEM lanes; when fewer rows are real, the digit slices of A are stored
// row-blocks apart in one region: the MMA reading slice t sees slices t+1.. in the rows
// beyond, which only feed accumulator rows nobody reads.
#include <type_traits>

#include "oz.cuh"

namespace w90g {

namespace {

constexpr int kS8 = 8;   // digits per operand in this kernel

template <int WP>
struct ExpSmem {
  using L = TileSmem<WP>;
  static constexpr int CW = L::CW, KC = L::KC, NC = L::NC, NCH = L::NCH;
  static constexpr int A_ROWS = (kS8 - 1) * WP + kTileRows;      // overlapped slices
  static constexpr int A_SLICE = WP * KC * 2;                     // bytes between slices
  static constexpr int A_BYTES = A_ROWS * KC * 2;
  static constexpr int B_BYTES = NC * KC * 2;                     // per slice
  static constexpr int TMEM_COLS = (kS8 * NC <= 128) ? 128 : ((kS8 * NC <= 256) ? 256 : 512);
  // W <= 32: the accumulators are staged through shared memory (aliasing the digit
  // slices, free once the MMAs are done) so that all warps recombine, not just the two
  // warps that can read the TMEM lanes of rows 0..31
  static constexpr bool STAGED = WP <= 32;
  static constexpr int STAGE_LD = NC + 1;                         // u32 row stride
  static constexpr size_t STAGE_BYTES = STAGED ? (size_t)kS8 * WP * STAGE_LD * 4 : 0;
  static constexpr size_t DIGIT_BYTES = (size_t)A_BYTES + (size_t)kS8 * B_BYTES;
  static constexpr size_t REGION = DIGIT_BYTES > STAGE_BYTES ? DIGIT_BYTES : STAGE_BYTES;
  static constexpr bool MATS_IN_SMEM = WP <= 32;
  static constexpr size_t MAT_BYTES = (size_t)WP * WP * 16;
  static constexpr size_t BYTES = REGION + (MATS_IN_SMEM ? 6 * MAT_BYTES : 0) + 1024;
};

__device__ __forceinline__ double cta_max(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// per-CTA state of the tensor product
struct OzCtx {
  unsigned char* sA;
  unsigned char* sB;
  uint32_t tmem;
  uint32_t mbar;
  uint32_t phase;
  int* rowexp;   // [WP]
  int* colexp;   // [WP]
  int* bad;
};

// Scale records of the chain's matrices: for every row and column the key of its largest
// |re| or |im| (0 for none, else the biased exponent + 1; the exponent above that value
// is key - 1023, as exp_above_bits gives it).  The epilogue that writes a matrix forms its
// record with shared-memory maxima, so that the products reading the matrix take their
// scales from shared memory instead of a pass over the operand.
__device__ __forceinline__ unsigned scale_key(double re, double im) {
  const unsigned long long ab = max(abs_bits(re), abs_bits(im));
  return ab ? (unsigned)(ab >> 52) + 1u : 0u;
}
__device__ __forceinline__ int key_exp(unsigned key) { return key ? (int)key - 1023 : 0; }

struct Rec {
  unsigned* row;
  unsigned* col;
};

// Power-of-two scales of a product: the exponent above the largest |re| or |im| of every
// row of A and every column of B, from the operands' records where given (arow / bcol),
// else by a pass over them.  The 2 WP rows / columns share the CTA's 256 threads (TPI
// consecutive lanes each, then a max across those lanes), so each thread reads W / TPI
// entries instead of W; the maximum does not depend on the order.
template <int WP>
__device__ __forceinline__ void ab_exponents(OzCtx& cx, const double2* A, const unsigned* arow,
                                             const double2* B, const unsigned* bcol, int W) {
  constexpr int ITEMS = 2 * WP;
  constexpr int TPI = ITEMS >= 256 ? 1 : (256 / ITEMS > 32 ? 32 : 256 / ITEMS);
  if (arow != nullptr && bcol != nullptr) {
    for (int i = threadIdx.x; i < ITEMS; i += blockDim.x)
      (i < WP ? cx.rowexp : cx.colexp)[i % WP] = key_exp(i < WP ? arow[i] : bcol[i - WP]);
    return;
  }
  for (int base = 0; base < ITEMS * TPI; base += blockDim.x) {
    const int gi = base + (int)threadIdx.x;
    const int idx = gi / TPI, sub = gi % TPI;
    const int r = idx % WP;
    const bool row_of_a = idx < WP;
    const unsigned* rec = row_of_a ? arow : bcol;
    unsigned long long mx = 0ull;
    if (idx < ITEMS && r < W && rec == nullptr) {
      // eight independent loads per round (the matrices may sit in L2), then the max
      for (int l0 = sub; l0 < W; l0 += 8 * TPI) {
        double2 v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int l = l0 + i * TPI;
          v[i] = (l < W) ? (row_of_a ? A[(size_t)l * W + r] : B[(size_t)r * W + l]) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) mx = max(mx, max(abs_bits(v[i].x), abs_bits(v[i].y)));
      }
    }
#pragma unroll
    for (int o = 1; o < TPI; o <<= 1)
      mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mx, o));
    if (idx < ITEMS && sub == 0)
      (row_of_a ? cx.rowexp : cx.colexp)[r] = rec != nullptr ? key_exp(rec[r]) : exp_above_bits(mx);
  }
}

// Where a product's result goes: `out`, made exactly Hermitian (sym = +1) or
// anti-Hermitian (sym = -1) from its upper triangle as the FP64 path's structured products
// produce it, or plain (sym = 0) with an elementwise term added (Add), and its scale
// record formed in `rec` (rec.row == nullptr: none).
struct Epi {
  double2* out;
  int sym;
  Rec rec;
};

// no elementwise term
struct NoAdd {
  static constexpr bool kActive = false;
  __device__ double2 operator()(int) const { return make_double2(0.0, 0.0); }
};

// block q of the Paterson-Stockmeyer polynomial, added by a Horner step's epilogue
template <class F>
struct HornerAdd {
  static constexpr bool kActive = true;
  const F* f;
  int q;
  __device__ double2 operator()(int e) const { return (*f)(q, e); }
};

__device__ __forceinline__ void rec_clear(const Rec& r, int n) {
  if (r.row != nullptr)
    for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) (i < n ? r.row : r.col)[i % n] = 0u;
}

// Adds the key of v (at row i, column j) to the record (shared-memory maxima).  (A warp
// maximum before one atomic per distinct index measured slower than these atomics.)
__device__ __forceinline__ void rec_add(const Rec& r, int i, int j, double2 v) {
  if (r.row != nullptr) {
    const unsigned key = scale_key(v.x, v.y);
    if (key) {
      atomicMax(r.row + i, key);
      atomicMax(r.col + j, key);
    }
  }
}

// Applies an Epi to a product already in C (the product forms whose epilogue does not
// apply it directly): out[e] from C[e] (its upper triangle when sym != 0) plus add(e),
// and the record.  out may be C.  All threads call.
template <int WP, class Add>
__device__ void epi_apply(const double2* C, const Epi& ep, const Add& add, int W) {
  if (ep.sym == 0 && !Add::kActive && ep.rec.row == nullptr && ep.out == C) return;
  rec_clear(ep.rec, WP);
  __syncthreads();
#pragma unroll 4
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
    const int i = e % W, j = e / W;
    double2 v;
    bool write = ep.out != C || Add::kActive;
    if (ep.sym != 0 && i > j) {
      const double2 u = C[(size_t)i * W + j];
      v = cmk(ep.sym * u.x, -ep.sym * u.y);
      write = true;
    } else if (ep.sym != 0 && i == j) {
      const double2 d = C[e];
      v = (ep.sym > 0) ? cmk(d.x, 0.0) : cmk(0.0, d.y);
      write = true;
    } else {
      v = C[e];
    }
    if (Add::kActive) v = cadd(v, add(e));
    if (write) ep.out[e] = v;
    rec_add(ep.rec, i, j, v);
  }
  __syncthreads();
}

// C = A B for W x W complex column-major matrices (generic pointers; C must not alias
// A or B), then the Epi applied from C.  All threads call; returns false (uniformly) if
// an MMA wait timed out.
template <int WP, class Add>
__device__ bool oz_cmm(OzCtx& cx, double2* C, const double2* A, const unsigned* arow, const double2* B,
                       const unsigned* bcol, int W, const Epi& ep, const Add& add) {
  using E = ExpSmem<WP>;
  constexpr int CW = E::CW, KC = E::KC, NC = E::NC, NCH = E::NCH;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // ---- power-of-two scales: rows of A, columns of B (over re and im parts)
  ab_exponents<WP>(cx, A, arow, B, bcol, W);
  __syncthreads();
  bool ok = true;
  for (int nc = 0; nc < NCH && ok; ++nc) {
    for (int kc = 0; kc < NCH && ok; ++kc) {
      // ---- A chunk: rows r < WP, complex K index l < CW -> real columns l, l + CW
      for (int e = tid; e < WP * CW; e += blockDim.x) {
        const int r = e % WP, l = e / WP;
        const int m = kc * CW + l;
        double2 a = make_double2(0.0, 0.0);
        if (r < W && m < W) a = A[(size_t)m * W + r];
        int xr[kS8], xi[kS8];
        const int ex = cx.rowexp[r];
        digits8(scaled_int56(a.x, ex), xr);
        digits8(scaled_int56(a.y, ex), xi);
        const uint32_t o_re = kmaj_off(r, l, KC), o_im = kmaj_off(r, l + CW, KC);
#pragma unroll
        for (int t = 0; t < kS8; ++t) {
          *(uint16_t*)(cx.sA + (size_t)t * E::A_SLICE + o_re) = int_to_bf16(xr[t]);
          *(uint16_t*)(cx.sA + (size_t)t * E::A_SLICE + o_im) = int_to_bf16(xi[t]);
        }
      }
      // ---- B chunk, embedded [[B_r, B_i], [-B_i, B_r]] stored as B^T (K-major):
      // row = real N index (c | c + CW), column = real K index (l | l + CW)
      for (int e = tid; e < CW * CW; e += blockDim.x) {
        const int l = e % CW, c = e / CW;
        const int mm = kc * CW + l, cc = nc * CW + c;
        double2 b = make_double2(0.0, 0.0);
        if (mm < W && cc < W) b = B[(size_t)cc * W + mm];
        int xr[kS8], xi[kS8];
        const int ex = cx.colexp[cc < WP ? cc : 0];
        digits8(scaled_int56(b.x, ex), xr);
        digits8(scaled_int56(b.y, ex), xi);
        const uint32_t o00 = kmaj_off(c, l, KC), o01 = kmaj_off(c + CW, l, KC);
        const uint32_t o10 = kmaj_off(c, l + CW, KC), o11 = kmaj_off(c + CW, l + CW, KC);
#pragma unroll
        for (int t = 0; t < kS8; ++t) {
          unsigned char* sb = cx.sB + (size_t)t * E::B_BYTES;
          *(uint16_t*)(sb + o00) = int_to_bf16(xr[t]);    // (K re, N re) =  B_r
          *(uint16_t*)(sb + o01) = int_to_bf16(xi[t]);    // (K re, N im) =  B_i
          *(uint16_t*)(sb + o10) = int_to_bf16(-xi[t]);   // (K im, N re) = -B_i
          *(uint16_t*)(sb + o11) = int_to_bf16(xr[t]);    // (K im, N im) =  B_r
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // descriptors from a base plus offsets / 16 (shared-memory addresses stay below
        // 2^18); B's digit planes follow one another as row groups of one K-major operand
        // and diagonal d's accumulator columns follow d - 1's, so slice t of A against
        // planes u0 .. u0 + n - 1 of B is one MMA with N = n NC (<= 256)
        const uint64_t da = smem_desc(smem_u32(cx.sA), 128, (KC / 8) * 128);
        const uint64_t db = smem_desc(smem_u32(cx.sB), 128, (KC / 8) * 128);
        constexpr int PPM = 256 / NC;
#pragma unroll
        for (int t = 0; t < kS8; ++t) {
#pragma unroll
          for (int u0 = 0; u0 + t <= kS8 - 1; u0 += PPM) {
            const int n = (kS8 - t - u0) < PPM ? (kS8 - t - u0) : PPM;
            const uint32_t dtm = cx.tmem + (uint32_t)((t + u0) * NC);
            const bool first_pair = (kc == 0) && (t == 0);
#pragma unroll
            for (int ks = 0; ks < KC / 16; ++ks) {
              const uint64_t ad = da + (uint64_t)(((size_t)t * E::A_SLICE + ks * 256) >> 4);
              const uint64_t bd = db + (uint64_t)(((size_t)u0 * E::B_BYTES + ks * 256) >> 4);
              const uint32_t acc = (first_pair && ks == 0) ? 0u : 1u;
              asm volatile(
                  "{\n\t.reg .pred p;\n\t"
                  "setp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                  :: "r"(dtm), "l"(ad), "l"(bd), "r"(idesc_bf16(n * NC)), "r"(acc)
                  : "memory");
            }
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     :: "r"(cx.mbar) : "memory");
      }
      // one thread waits for the commit (the others wait at the CTA barrier, issuing nothing)
      if (tid == 0 && !mbar_wait(cx.mbar, cx.phase)) {
        // record the error; drain the MMAs before tensor memory or the operands are reused
        *cx.bad = 1;
        mbar_drain(cx.mbar, cx.phase);
      }
      cx.phase ^= 1u;
      __syncthreads();
      ok = (*cx.bad == 0);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (!ok) break;
    // C(r, c) = (sum_d D_d 2^(7(7-d))) 2^(rowexp + colexp - 63), exact in 128 bits
    auto recombine = [&](const uint32_t* dr, const uint32_t* di, int stride, int r, int c) {
      __int128 sr = float_to_int_exact24(__uint_as_float(dr[0]));
      __int128 si = float_to_int_exact24(__uint_as_float(di[0]));
#pragma unroll
      for (int d = 1; d < kS8; ++d) {
        sr = (sr << 7) + float_to_int_exact24(__uint_as_float(dr[d * stride]));
        si = (si << 7) + float_to_int_exact24(__uint_as_float(di[d * stride]));
      }
      const int sc = cx.rowexp[r] + cx.colexp[c] - 63;
      C[(size_t)c * W + r] = make_double2(int128_scaled_to_double(sr, sc), int128_scaled_to_double(si, sc));
    };
    const int wq = warp & 3, half = warp >> 2;
    const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
    const int jbeg = half * (CW / 2), jend = jbeg + CW / 2;
    if (E::STAGED) {
      // ---- TMEM -> shared (warps 0 and 4 hold rows 0..31), then all warps recombine
      uint32_t* stage = (uint32_t*)cx.sA;
      if (wq == 0) {
#pragma unroll 1
        for (int j0 = jbeg; j0 < jend; j0 += 4) {
#pragma unroll
          for (int d = 0; d < kS8; ++d) {
            uint32_t q[4], s4[4];
            const uint32_t ta = cx.tmem + lane_base + (uint32_t)(d * NC + j0);
            const uint32_t tb = cx.tmem + lane_base + (uint32_t)(d * NC + CW + j0);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]) : "r"(ta));
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(s4[0]), "=r"(s4[1]), "=r"(s4[2]), "=r"(s4[3]) : "r"(tb));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (lane < WP) {
              uint32_t* row = stage + ((size_t)d * WP + lane) * E::STAGE_LD;
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                row[j0 + j] = q[j];
                row[CW + j0 + j] = s4[j];
              }
            }
          }
        }
      }
      __syncthreads();
      for (int e = tid; e < W * CW; e += blockDim.x) {
        const int r = e % W, j = e / W;
        const int c = nc * CW + j;
        if (c >= W) continue;
        const uint32_t* rowp = stage + (size_t)r * E::STAGE_LD;
        recombine(rowp + j, rowp + CW + j, WP * E::STAGE_LD, r, c);
      }
    } else {
      // ---- direct: TMEM lane r = row r; warps w and w+4 split the chunk's columns
      const int r = wq * 32 + lane;
      if (wq * 32 < W) {   // warp-uniform
#pragma unroll 1
        for (int j0 = jbeg; j0 < jend; j0 += 4) {
          uint32_t q[kS8][4], s4[kS8][4];
#pragma unroll
          for (int d = 0; d < kS8; ++d) {
            const uint32_t ta = cx.tmem + lane_base + (uint32_t)(d * NC + j0);
            const uint32_t tb = cx.tmem + lane_base + (uint32_t)(d * NC + CW + j0);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(q[d][0]), "=r"(q[d][1]), "=r"(q[d][2]), "=r"(q[d][3])
                         : "r"(ta));
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(s4[d][0]), "=r"(s4[d][1]), "=r"(s4[d][2]), "=r"(s4[d][3])
                         : "r"(tb));
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (r < W) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int c = nc * CW + j0 + j;
              if (c < W) recombine(&q[0][j], &s4[0][j], 4, r, c);
            }
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  __syncthreads();
  if (ok) epi_apply<WP>(C, ep, add, W);
  return ok;
}

// ---------------------------------------------------------------------------
// Second product form (num_wann <= 64): C = A B through
//     [C_r; C_i] = [[A_r, -A_i], [A_i, A_r]] [B_r; B_i]
// i.e. 2W accumulator rows (real parts in rows 0..WP-1, imaginary parts in rows
// WP..2WP-1), N = W columns, K = 2W; operands split into 7 signed 8-bit digits (56 bits;
// exact FP16 values, built two at a time by a packed FP16 subtraction) and the 28 digit
// pairs with t+u <= 6 kept.  Against the first
// form this halves N and TMEM, drops 36 pairs to 28 at the same 56-bit precision, and
// (FP64 matrices in L2 instead of shared memory) lets two CTAs share an SM.  Exactness:
// a diagonal holds at most 7 pairs of products <= 2^14 over K <= 128 terms, < 2^24.
// ---------------------------------------------------------------------------
constexpr int kS2 = 7;

template <int WP, bool SMEM_MATS = false>
struct Exp2Smem {
  static constexpr int CW = WP < 32 ? WP : 32;      // complex inner indices per K chunk
  static constexpr int KC = 2 * CW;                 // real K per chunk
  static constexpr int NCHK = WP / CW;              // K chunks
  static constexpr int ROWS = 2 * WP;               // accumulator rows
  static constexpr int N = WP < 16 ? 16 : WP;       // accumulator columns (MMA N >= 16)
  static constexpr int A_SLICE = ROWS * KC * 2;     // bytes between the overlapped slices
  static constexpr int A_BYTES = (kS2 - 1) * A_SLICE + kTileRows * KC * 2;
  static constexpr int B_BYTES = N * KC * 2;        // per slice
  static constexpr int TMEM_COLS = (kS2 * N <= 128) ? 128 : ((kS2 * N <= 256) ? 256 : 512);
  static constexpr bool STAGED = ROWS <= 64;        // rows in TMEM subpartitions 0-1 only
  static constexpr int STAGE_LD = N + 1;
  static constexpr size_t STAGE_BYTES = STAGED ? (size_t)kS2 * ROWS * STAGE_LD * 4 : 0;
  static constexpr size_t DIGIT_BYTES = (size_t)A_BYTES + (size_t)kS2 * B_BYTES;
  static constexpr size_t REGION = DIGIT_BYTES > STAGE_BYTES ? DIGIT_BYTES : STAGE_BYTES;
  // the six FP64 matrices of the exp chain in shared memory: always for WP <= 16; for
  // WP = 32 on request (one CTA per SM then, shared-memory latency for every operand read)
  static constexpr bool MATS_IN_SMEM = WP <= 16 || SMEM_MATS;
  static constexpr size_t MAT_BYTES = (size_t)WP * WP * 16;
  static constexpr size_t NEED = REGION + (MATS_IN_SMEM ? 6 * MAT_BYTES : 0) + 1024;
  // never more CTAs on an SM than its 512 TMEM columns hold: request enough shared
  // memory that (512 / TMEM_COLS + 1) CTAs cannot fit in the SM's 228 KB
  static constexpr size_t FLOOR = 233472 / (512 / TMEM_COLS + 1) - 1024 + 16;
  static constexpr size_t BYTES = NEED > FLOOR ? NEED : FLOOR;
};

// Part (0 re, 1 im) of 8 values base[(m0 + i) * stride], i < 8 (zero where m0 + i >= W or
// !valid): the operand run a thread slices.
__device__ __forceinline__ void load_run8(double (&v)[8], const double2* base, size_t stride, int m0, int W,
                                          bool valid, int part) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int m = m0 + i;
    v[i] = 0.0;
    if (valid && m < W) v[i] = ((const double*)(base + (size_t)m * stride))[part];
  }
}

// The seven 8-bit digit planes of the 8 values scaled by 2^(55 - ex), as packed FP16
// pairs: w[t][i / 2] holds digit t of values i (low half) and i + 1 -- the digits of
// digits7x8, without its serial recoding.  With C = 128 (1 + 2^8 + ... + 2^40), byte t' of
// N + C is digit 6 - t' plus 128 (adding 128 at every lower byte position turns the
// centred digits into the plain bytes of N + C: x_6 = sext8(N mod 2^8) = byte0(N + 128) -
// 128, and (N - x_6) / 2^8 = (N + 128) >> 8, so the next step repeats on N + 128 shifted),
// and the top digit is (N + C) >> 48 (arithmetic), so b = digit + 128 lies in [0, 256].
// With 0x6400 above it, b is the FP16 number 1024 + b: one byte permute, one mask and one
// packed subtraction of 1152 give two digits.  Exact: FP16 holds the integers to 2048, and
// the difference of two of them is rounded to itself.
__device__ __forceinline__ void slice_run8_h(uint32_t (&w)[7][4], const double (&v)[8], int ex) {
#pragma unroll
  for (int i = 0; i < 8; i += 2) {
    const long long ma = scaled_int55(v[i], ex) + 0x808080808080LL;
    const long long mb = scaled_int55(v[i + 1], ex) + 0x808080808080LL;
    const uint32_t la = (uint32_t)ma, lb = (uint32_t)mb;
    const uint32_t ha = (uint32_t)((unsigned long long)ma >> 32), hb = (uint32_t)((unsigned long long)mb >> 32);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const uint32_t bt = (uint32_t)(t & 3);
      const uint32_t sel = bt | (bt << 4) | ((4u + bt) << 8) | ((4u + bt) << 12);
      const uint32_t p = __byte_perm(t < 4 ? la : ha, t < 4 ? lb : hb, sel);
      w[6 - t][i >> 1] = f16x2_sub((p & 0x00FF00FFu) | 0x64006400u, 0x64806480u);
    }
    const uint32_t ta = (uint32_t)((int)(ma >> 48) + 128), tb = (uint32_t)((int)(mb >> 48) + 128);
    w[0][i >> 1] = f16x2_sub(ta | (tb << 16) | 0x64006400u, 0x64806480u);
  }
}

// -x for both halves of a packed FP16 pair (a zero becomes -0, the same in every product)
__device__ __forceinline__ uint32_t f16x2_neg(uint32_t w) { return w ^ 0x80008000u; }

// C = A B, then the Epi.  num_wann <= 32 (staged accumulators): the epilogue applies the
// Epi itself and writes ep.out only (C unused; ep.out may alias B, whose digits are in
// shared memory before the MMAs run, but not A); WP = 64: C as in oz_cmm.
template <int WP, class Add>
__device__ bool oz_cmm2(OzCtx& cx, double2* C, const double2* A, const unsigned* arow, const double2* B,
                        const unsigned* bcol, int W, const Epi& ep, const Add& add) {
  using E = Exp2Smem<WP>;
  constexpr int CW = E::CW, KC = E::KC, N = E::N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  ab_exponents<WP>(cx, A, arow, B, bcol, W);
  __syncthreads();
  bool ok = true;
  for (int kc = 0; kc < E::NCHK && ok; ++kc) {
    // ---- A_emb chunk: complex (r, l) -> rows r (re) and WP + r (im), K l (re) / CW + l (im),
    // and B_emb chunk as B^T (K-major): row = output column c, K l (re) / CW + l (im).  A
    // thread slices one part (re or im) of 8 consecutive l of a row of A and of a column of
    // B (contiguous in memory) -- a whole 16-byte core-matrix row per digit plane -- with
    // both runs' loads issued before either is sliced.  The A part goes to both places it
    // occupies (A_r: (re, K re) and (im, K im); A_i: (im, K re) and, negated, (re, K im));
    // lanes take consecutive rows / columns, so the 16-byte stores do not conflict.
    {
      constexpr int LG = CW / 8, NIA = WP * LG * 2, NIB = N * LG * 2;
      constexpr int NI = NIA > NIB ? NIA : NIB;
      for (int it = tid; it < NI; it += 256) {
        const int r = it % WP, lga = (it / WP) % LG, pa = it / (WP * LG);
        const int c = it % N, lgb = (it / N) % LG, pb = it / (N * LG);
        double va[8], vb[8];
        if (it < NIA) load_run8(va, A + r, (size_t)W, kc * CW + lga * 8, W, r < W, pa);
        if (it < NIB) load_run8(vb, B + (size_t)c * W, (size_t)1, kc * CW + lgb * 8, W, c < W, pb);
        uint32_t w[kS2][4];
        if (it < NIA) {
          slice_run8_h(w, va, cx.rowexp[r]);
          const int kq = lga * 8;
          const uint32_t o1 = pa == 0 ? kmaj_off(r, kq, KC) : kmaj_off(WP + r, kq, KC);
          const uint32_t o2 = pa == 0 ? kmaj_off(WP + r, CW + kq, KC) : kmaj_off(r, CW + kq, KC);
#pragma unroll
          for (int t = 0; t < kS2; ++t) {
            unsigned char* sa = cx.sA + (size_t)t * E::A_SLICE;
            *(uint4*)(sa + o1) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
            *(uint4*)(sa + o2) = pa == 0 ? make_uint4(w[t][0], w[t][1], w[t][2], w[t][3])
                                         : make_uint4(f16x2_neg(w[t][0]), f16x2_neg(w[t][1]),
                                                      f16x2_neg(w[t][2]), f16x2_neg(w[t][3]));
          }
        }
        if (it < NIB) {
          slice_run8_h(w, vb, cx.colexp[c < WP ? c : 0]);
          const uint32_t o = kmaj_off(c, pb * CW + lgb * 8, KC);
#pragma unroll
          for (int t = 0; t < kS2; ++t)
            *(uint4*)(cx.sB + (size_t)t * E::B_BYTES + o) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // descriptors of the slices' K-steps: the base descriptor plus the byte offset / 16 in
      // its address field (shared-memory addresses stay below 2^18, so the field holds it)
      const uint64_t da = smem_desc(smem_u32(cx.sA), 128, (KC / 8) * 128);
      const uint64_t db = smem_desc(smem_u32(cx.sB), 128, (KC / 8) * 128);
      // B's digit planes follow one another as row groups of one K-major operand and
      // diagonal d's accumulator columns follow d - 1's: slice t of A against planes
      // u0 .. u0 + n - 1 of B is one MMA with N = n N, writing diagonals t + u0 .. (N <= 256)
      constexpr int PPM = 256 / N;
#pragma unroll
      for (int t = 0; t < kS2; ++t) {
#pragma unroll
        for (int u0 = 0; u0 + t <= kS2 - 1; u0 += PPM) {
          const int n = (kS2 - t - u0) < PPM ? (kS2 - t - u0) : PPM;
          const uint32_t dtm = cx.tmem + (uint32_t)((t + u0) * N);
          const bool first_pair = (kc == 0) && (t == 0);
#pragma unroll
          for (int ks = 0; ks < KC / 16; ++ks) {
            const uint64_t ad = da + (uint64_t)(((size_t)t * E::A_SLICE + ks * 256) >> 4);
            const uint64_t bd = db + (uint64_t)(((size_t)u0 * E::B_BYTES + ks * 256) >> 4);
            const uint32_t acc = (first_pair && ks == 0) ? 0u : 1u;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                :: "r"(dtm), "l"(ad), "l"(bd), "r"(idesc_f16(n * N)), "r"(acc)
                : "memory");
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                   :: "r"(cx.mbar) : "memory");
    }
    // one thread waits for the commit (the others wait at the CTA barrier, issuing nothing)
    if (tid == 0 && !mbar_wait(cx.mbar, cx.phase)) {
      *cx.bad = 1;
      mbar_drain(cx.mbar, cx.phase);
    }
    cx.phase ^= 1u;
    __syncthreads();
    ok = (*cx.bad == 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (ok) {
    // accumulator row `row` (part = row / WP: 0 real, 1 imaginary; rr = row % WP),
    // column c: sum_d D_d 2^(8(6-d)) 2^(rowexp + colexp - 62)
    auto recombine = [&](const uint32_t* dd, int stride, int row, int c) {
      const int rr = row % WP;
      const double v = recombine7x8(dd, stride, cx.rowexp[rr] + cx.colexp[c] - 62);
      double* dst = (double*)(C + (size_t)c * W + rr);
      dst[row / WP] = v;
    };
    const int wq = warp & 3, half = warp >> 2;
    const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
    constexpr int NH = N / 2;   // columns per warp half
    if (E::STAGED) {
      rec_clear(ep.rec, WP);     // the operands' scales are in cx already
      uint32_t* stage = (uint32_t*)cx.sA;
      if (wq * 32 < E::ROWS) {
#pragma unroll 1
        for (int j0 = half * NH; j0 < (half + 1) * NH; j0 += 4) {
          uint32_t q[kS2][4];
#pragma unroll
          for (int d = 0; d < kS2; ++d)
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(q[d][0]), "=r"(q[d][1]), "=r"(q[d][2]), "=r"(q[d][3])
                         : "r"(cx.tmem + lane_base + (uint32_t)(d * N + j0)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          const int row = wq * 32 + lane;
          if (row < E::ROWS) {
#pragma unroll
            for (int d = 0; d < kS2; ++d) {
              uint32_t* rp = stage + ((size_t)d * E::ROWS + row) * E::STAGE_LD + j0;
              rp[0] = q[d][0];
              rp[1] = q[d][1];
              rp[2] = q[d][2];
              rp[3] = q[d][3];
            }
          }
        }
      }
      __syncthreads();
      // both parts of element (rr, c) by one thread
      auto element = [&](int rr, int c) -> double2 {
        const int sc = cx.rowexp[rr] + cx.colexp[c] - 62;
        const double re = recombine7x8(stage + (size_t)rr * E::STAGE_LD + c, E::ROWS * E::STAGE_LD, sc);
        const double im = recombine7x8(stage + (size_t)(WP + rr) * E::STAGE_LD + c, E::ROWS * E::STAGE_LD, sc);
        return make_double2(re, im);
      };
      if (ep.sym == 0) {
#pragma unroll 2
        for (int e = tid; e < W * W; e += blockDim.x) {
          const int rr = e % W, c = e / W;
          double2 v = element(rr, c);
          if (Add::kActive) v = cadd(v, add(e));
          ep.out[e] = v;
          rec_add(ep.rec, rr, c, v);
        }
      } else {
        // the upper triangle rr <= c (linear index e = c (c + 1) / 2 + rr), mirrored
        const int ntri = W * (W + 1) / 2;
        for (int e = tid; e < ntri; e += blockDim.x) {
          int c = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
          while (c * (c + 1) / 2 > e) --c;
          while ((c + 1) * (c + 2) / 2 <= e) ++c;
          const int rr = e - c * (c + 1) / 2;
          double2 v = element(rr, c);
          if (rr == c) {
            v = (ep.sym > 0) ? cmk(v.x, 0.0) : cmk(0.0, v.y);
            ep.out[(size_t)c * W + c] = v;
            rec_add(ep.rec, c, c, v);
          } else {
            ep.out[(size_t)c * W + rr] = v;
            const double2 m = cmk(ep.sym * v.x, -ep.sym * v.y);
            ep.out[(size_t)rr * W + c] = m;
            rec_add(ep.rec, rr, c, v);
            // (a record whose rows and columns share one array already holds the mirror)
            if (ep.rec.row != ep.rec.col) rec_add(ep.rec, c, rr, m);
          }
        }
      }
    } else {
      const int row = wq * 32 + lane;   // all 128 lanes hold rows (ROWS = 128)
      const int rr = row % WP;
#pragma unroll 1
      for (int j0 = half * NH; j0 < (half + 1) * NH; j0 += 4) {
        uint32_t q[kS2][4];
#pragma unroll
        for (int d = 0; d < kS2; ++d)
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                       : "=r"(q[d][0]), "=r"(q[d][1]), "=r"(q[d][2]), "=r"(q[d][3])
                       : "r"(cx.tmem + lane_base + (uint32_t)(d * N + j0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (rr < W) {
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (j0 + j < W) recombine(&q[0][j], 4, row, j0 + j);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (ok && !E::STAGED) epi_apply<WP>(C, ep, add, W);
  return ok;
}

// product policies of the exp kernel: first form for WP = 128, second for WP <= 64
template <int WP>
struct ProdV1 {
  using E = ExpSmem<WP>;
  static constexpr int TMEM_COLS = E::TMEM_COLS;
  static constexpr bool MATS_IN_SMEM = E::MATS_IN_SMEM;
  static constexpr size_t REGION = E::REGION, BYTES = E::BYTES;
  static constexpr size_t SB_OFFSET = E::A_BYTES;
  template <class Add>
  __device__ static bool mm(OzCtx& cx, double2* C, const double2* A, const unsigned* arow, const double2* B,
                            const unsigned* bcol, int W, const Epi& ep, const Add& add) {
    return oz_cmm<WP>(cx, C, A, arow, B, bcol, W, ep, add);
  }
};

template <int WP, bool SMEM_MATS = false>
struct ProdV2 {
  using E = Exp2Smem<WP, SMEM_MATS>;
  static constexpr int TMEM_COLS = E::TMEM_COLS;
  static constexpr bool MATS_IN_SMEM = E::MATS_IN_SMEM;
  static constexpr size_t REGION = E::REGION, BYTES = E::BYTES;
  static constexpr size_t SB_OFFSET = E::A_BYTES;
  template <class Add>
  __device__ static bool mm(OzCtx& cx, double2* C, const double2* A, const unsigned* arow, const double2* B,
                            const unsigned* bcol, int W, const Epi& ep, const Add& add) {
    return oz_cmm2<WP>(cx, C, A, arow, B, bcol, W, ep, add);
  }
};

template <int WP, bool SMEM_MATS = false>
using ExpProd = typename std::conditional<(WP <= 64), ProdV2<WP, SMEM_MATS>, ProdV1<WP>>::type;

// x 2^-j (sc = 2^-j): an exponent subtraction where the result is a normal number (the
// product is exact there, so the bits are those of x * sc), else the FP64 multiply
__device__ __forceinline__ double scale_pow2(double x, int j, double sc) {
  const long long b = __double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7FF);
  if (be > j && be != 0x7FF) return __longlong_as_double(b - ((long long)j << 52));
  return x * sc;
}

// The number of halvings that bring v >= 0 to theta (a positive normal) or below, at most
// 60: the count of the loop "while (v > theta && j < 60) { v *= 0.5; ++j; }" (halving is
// exact), from the bits with integer ops only.  Non-negative doubles order like their bit
// patterns; with v = mv 2^ev and theta = mt 2^et (mantissas in [1, 2)), v 2^-j <= theta
// first holds at j = ev - et, or one later where mv > mt.  (0 for nan, where v > theta is
// false; 60 for inf.)
__device__ __forceinline__ int halvings(double v, double theta) {
  constexpr long long kMant = 0x000FFFFFFFFFFFFFLL;
  const long long vb = __double_as_longlong(v), tb = __double_as_longlong(theta);
  if (vb <= tb) return 0;
  if ((vb >> 52) == 0x7FF && (vb & kMant) != 0) return 0;
  const int j = (int)(vb >> 52) - (int)(tb >> 52) + ((vb & kMant) > (tb & kMant) ? 1 : 0);
  return j > 60 ? 60 : j;
}

// Degree m, block size pw and squarings js of exp(X) from its 1-norm, with the cost in
// products (powers plus Horner steps, plus js): the FP64 path's table (k_exp_u), the
// cheapest candidate after the halvings that bring the norm under its theta.
struct ExpPlan {
  int m, pw, js, cost;
};
__device__ const int kPlanM[5] = {4, 6, 8, 12, 16};
__device__ const int kPlanP[5] = {4, 3, 4, 4, 4};
__device__ const double kPlanTheta[5] = {1.6e-3, 1.68e-2, 6.6e-2, 0.32, 0.78};
__device__ const int kPlanCost[5] = {3, 3, 4, 5, 6};

__device__ __noinline__ ExpPlan exp_plan(double nrm) {
  ExpPlan pl{16, 4, 0, 1 << 30};
  for (int c = 0; c < 5; ++c) {
    const int j = halvings(nrm, kPlanTheta[c]);
    const int cost = kPlanCost[c] + j;
    if (cost < pl.cost) pl = ExpPlan{kPlanM[c], kPlanP[c], j, cost};
  }
  return pl;
}

// Whether every norm within a relative 2^-14 of nrm gets the same halvings for every
// candidate -- nrm finite and at least that far from each candidate's boundaries theta
// 2^(j-1) and theta 2^j -- so that an estimate of the norm to that accuracy picks the plan
// the exact norm picks.  (nrm < x 2^j compares the bits of nrm with those of x plus j in
// the exponent field, x 2^j being a normal number here.)
__device__ __noinline__ bool exp_plan_stable(double nrm) {
  if (!(nrm < 1e300)) return false;
  const long long nb = __double_as_longlong(nrm);
  for (int c = 0; c < 5; ++c) {
    const double th = kPlanTheta[c];
    const int j = halvings(nrm, th);
    const long long lo = __double_as_longlong(th * (1.0 - 0x1p-14)), hi = __double_as_longlong(th * (1.0 + 0x1p-14));
    if (j < 60 && !(nb < lo + ((long long)j << 52))) return false;
    if (j > 0 && !(nb > hi + ((long long)(j - 1) << 52))) return false;
  }
  return true;
}

// |re + i im| to a relative 2^-20 with no FP64 instruction: each part truncated to FP32
// through its bits (0 below 2^-60, +inf above 2^60 or for inf / nan), then FP32 fma and
// q rsqrt(q) (rsqrtf: 2 ulp).  A column sum of these (<= 128 terms, FP32) is within 2^-16
// of the FP64 one.  (An infinite estimate gives a nan norm, which is never stable.)
__device__ __forceinline__ float abs_est(double2 v) {
  auto f32 = [](double x) -> float {
    const unsigned long long b = abs_bits(x);
    const int e = (int)(b >> 52) - 1023;
    if (e < -60) return 0.0f;
    if (e > 60) return __int_as_float(0x7f800000);
    return __uint_as_float(((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
  };
  const float a = f32(v.x), b = f32(v.y);
  const float q = fmaf(a, a, b * b);
  return q > 0.0f ? q * rsqrtf(q) : 0.0f;
}

__device__ const double kOzInvFact[17] = {
    1.0, 1.0, 0.5, 1.6666666666666666e-01, 4.1666666666666664e-02, 8.3333333333333332e-03,
    1.3888888888888889e-03, 1.9841269841269841e-04, 2.4801587301587302e-05,
    2.7557319223985893e-06, 2.7557319223985888e-07, 2.5052108385441720e-08,
    2.0876756987868100e-09, 1.6059043836821613e-10, 1.1470745597729725e-11,
    7.6471637318198164e-13, 4.7794773323873853e-14};

}  // namespace

// which = 0: trial step (also forms D = coefG (G or Gp) + coefD D_prev); 1: optimal step
template <int WP, bool SMEM_MATS>
__global__ void __launch_bounds__(256, 2) k_oz_exp(const Problem* __restrict__ probs, WorkMap wm, int which) {
  using E = ExpProd<WP, SMEM_MATS>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_rowexp[WP], s_colexp[WP];
  __shared__ unsigned s_key[6][2][WP];
  __shared__ int s_bad;
  __shared__ double red[256];

  int k;
  const int p = locate(wm, blockIdx.x, k);
  const Problem& P = probs[p];
  CtrlState* st = P.st;
  if (st->done) return;
  if (which == 1 && !st->do_second) return;
  const int W = P.W, WW = W * W;
  const int tid = threadIdx.x, warp = tid >> 5;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(&tmem_slot)), "r"((uint32_t)E::TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_bad = 0;
  }
  // FP64 matrices: shared memory for WP <= 32, else the per-k workspace (6 W^2)
  double2* mats = E::MATS_IN_SMEM ? (double2*)(base + E::REGION)
                                  : (P.work + (size_t)k * 6 * WW);
  double2 *X = mats, *Y2 = mats + WW, *Y3 = mats + 2 * WW, *Y4 = mats + 3 * WW, *R = mats + 4 * WW,
          *T = mats + 5 * WW;
  double2* Dk = P.D + (size_t)k * WW;
  const double s = (which == 0) ? st->s_trial : st->s_second;
  // scale records of X, Y2, Y3, Y4, R, T (see Rec).  The powers are exactly Hermitian or
  // anti-Hermitian (|re| and |im| of element (i, j) are those of (j, i)), so row i and
  // column i of their records are the same maximum: one array serves both.
  Rec rX{s_key[0][0], s_key[0][1]}, rY2{s_key[1][0], s_key[1][0]}, rY3{s_key[2][0], s_key[2][0]},
      rY4{s_key[3][0], s_key[3][0]}, rR{s_key[4][0], s_key[4][1]}, rT{s_key[5][0], s_key[5][1]};
  rec_clear(rX, WP);
  // ---- X = s D (the trial step first forms D = coefG G + coefD D_prev; in the
  // symmetry-adapted mode k_sym_dir has formed D already) and estimates of the moduli
  // |X_ij| into shared scratch.  num_wann <= 32: X stays in registers (element tid + 256 i
  // in slot i) until it is scaled below.
  constexpr bool XREG = WP <= 32;
  constexpr int NE = XREG ? (WP * WP + 255) / 256 : 1;
  double2 xr[NE];
  // the digit region is free before the first product: |X_ij| estimates, then (where the
  // exact norm is needed, once the estimates are summed) the exact moduli in its place
  float* absf = (float*)base;
  double* absx = (double*)base;
  const bool form_d = (which == 0 && P.sym_nir == 0);
  const double cg = st->coefG, cd = st->coefD;
  const double2* Gk = form_d ? (st->use_gp ? P.pc_gp : P.G) + (size_t)k * WW : nullptr;
  // (each product and the sum rounded on its own, as the oracle forms D: no contraction
  // into an FMA, whose choice of product would follow the code's shape)
  auto form_x = [&](int e) -> double2 {
    double2 d = Dk[e];
    if (form_d) {
      const double2 g = Gk[e];
      d = cmk(__dadd_rn(__dmul_rn(g.x, cg), __dmul_rn(d.x, cd)), __dadd_rn(__dmul_rn(g.y, cg), __dmul_rn(d.y, cd)));
      Dk[e] = d;
    }
    const double2 x = cscale(d, s);
    absf[e] = abs_est(x);
    return x;
  };
  if (XREG) {
#pragma unroll
    for (int i = 0; i < NE; ++i) {
      const int e = tid + 256 * i;
      if (e < WW) xr[i] = form_x(e);
    }
  } else {
#pragma unroll 4
    for (int e = tid; e < WW; e += 256) X[e] = form_x(e);
  }
  __syncthreads();
  OzCtx cx{base, base + E::SB_OFFSET, tmem_slot, smem_u32(&mbar), 0u, s_rowexp, s_colexp, &s_bad};

  // ---- degree / squarings from the 1-norm (the FP64 path's table and choice, exp_plan).
  // The plan depends on the norm only through which side of each theta 2^j it lies, so
  // the FP32 estimate decides wherever it is clearly inside one interval
  // (exp_plan_stable); else the exact FP64 norm is formed -- moduli, then each column
  // summed in row order -- as the FP64 path forms it.  One thread plans, all read it.
  __shared__ float s_wmax[8];
  __shared__ int s_plan[5];
  {
    float colmax = 0.0f;
    for (int j = tid; j < W; j += 256) {
      float a = 0.0f;
      for (int i = 0; i < W; ++i) a += absf[(size_t)j * W + i];
      colmax = fmaxf(colmax, a);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) colmax = fmaxf(colmax, __shfl_xor_sync(0xffffffffu, colmax, o));
    if ((tid & 31) == 0) s_wmax[warp] = colmax;
  }
  __syncthreads();
  if (tid == 0) {
    float nf = 0.0f;
    for (int w = 0; w < 8; ++w) nf = fmaxf(nf, s_wmax[w]);
    const bool stable = exp_plan_stable((double)nf);
    const ExpPlan pl = exp_plan((double)nf);
    s_plan[0] = pl.m;
    s_plan[1] = pl.pw;
    s_plan[2] = pl.js;
    s_plan[3] = stable ? 0 : 1;
    s_plan[4] = pl.cost;
  }
  __syncthreads();
  if (s_plan[3]) {
    auto exact_abs = [&](int e, double2 x) { absx[e] = sqrt(cabs2(x)); };
    if (XREG) {
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        const int e = tid + 256 * i;
        if (e < WW) exact_abs(e, xr[i]);
      }
    } else {
      for (int e = tid; e < WW; e += 256) exact_abs(e, X[e]);
    }
    __syncthreads();
    double colmax = 0.0;
    for (int j = tid; j < W; j += 256) {
      double a = 0.0;
      for (int i = 0; i < W; ++i) a += absx[(size_t)j * W + i];
      colmax = fmax(colmax, a);
    }
    __syncthreads();
    const double nrm = cta_max(colmax, red);
    if (tid == 0) {
      const ExpPlan pl = exp_plan(nrm);
      s_plan[0] = pl.m;
      s_plan[1] = pl.pw;
      s_plan[2] = pl.js;
      s_plan[4] = pl.cost;
    }
    __syncthreads();
  }
  const int m = s_plan[0], pw = s_plan[1], js = s_plan[2];
  const double sc = ldexp(1.0, -js);
  auto scale_x = [&](int e, double2 x) {
    const double2 v = make_double2(scale_pow2(x.x, js, sc), scale_pow2(x.y, js, sc));
    X[e] = v;
    rec_add(rX, e % W, e / W, v);
  };
  if (XREG) {
#pragma unroll
    for (int i = 0; i < NE; ++i) {
      const int e = tid + 256 * i;
      if (e < WW) scale_x(e, xr[i]);
    }
  } else {
#pragma unroll 4
    for (int e = tid; e < WW; e += 256) scale_x(e, X[e]);
  }
  __syncthreads();
  const NoAdd none;
  // powers, exactly Hermitian (even) / anti-Hermitian (odd) as the FP64 path forms them
  bool ok = E::mm(cx, Y2, X, rX.row, X, rX.col, W, Epi{Y2, 1, rY2}, none);
  if (ok) ok = E::mm(cx, Y3, Y2, rY2.row, X, rX.col, W, Epi{Y3, -1, rY3}, none);
  if (ok && pw >= 4) ok = E::mm(cx, Y4, Y2, rY2.row, Y2, rY2.col, W, Epi{Y4, 1, rY4}, none);
  const double2* Yp = (pw == 4) ? Y4 : Y3;
  const Rec rYp = (pw == 4) ? rY4 : rY3;
  const int nblk = (m + pw) / pw;
  // block q of the polynomial, sum_r c_{pw q + r} X^r (X^0 = I), one FMA per term and part
  // (the FP64 pipe runs at 1/64 of FP32 on this chip: these elementwise terms are a large
  // part of the chain's FP64 work)
  auto blk = [&](int q, int e) -> double2 {
    const int i = e % W, j = e / W;
    double2 v = cmk(0.0, 0.0);
    for (int r = 0; r < pw; ++r) {
      const int deg = pw * q + r;
      if (deg > m) break;
      const double c = kOzInvFact[deg];
      if (r == 0) {
        if (i == j) v.x += c;
      } else {
        const double2 y = (r == 1) ? X[e] : ((r == 2) ? Y2[e] : Y3[e]);
        v = cmk(fma(y.x, c, v.x), fma(y.y, c, v.y));
      }
    }
    return v;
  };
  int q = nblk - 1;
  rec_clear(rR, WP);
  __syncthreads();
  if (pw * q == m) {
    const double cm = kOzInvFact[m];
    #pragma unroll 4
    for (int e = tid; e < WW; e += blockDim.x) {
      const double2 b = blk(q - 1, e), y = Yp[e];
      const double2 v = cmk(fma(y.x, cm, b.x), fma(y.y, cm, b.y));
      R[e] = v;
      rec_add(rR, e % W, e / W, v);
    }
    q -= 1;
  } else {
    #pragma unroll 4
    for (int e = tid; e < WW; e += blockDim.x) {
      const double2 v = blk(q, e);
      R[e] = v;
      rec_add(rR, e % W, e / W, v);
    }
  }
  __syncthreads();
  // Horner steps R <- Yp R + block q (the product's epilogue adds the block)
  for (q = q - 1; q >= 0 && ok; --q) {
    const HornerAdd<decltype(blk)> hadd{&blk, q};
    ok = E::mm(cx, T, Yp, rYp.row, R, rR.col, W, Epi{R, 0, rR}, hadd);
  }
  double2* a = R;
  double2* b = T;
  Rec ra = rR, rb = rT;
  for (int sq = 0; sq < js && ok; ++sq) {
    ok = E::mm(cx, b, a, ra.row, a, ra.col, W, Epi{b, 0, rb}, none);
    double2* tmp = a;
    a = b;
    b = tmp;
    const Rec rt = ra;
    ra = rb;
    rb = rt;
  }
  // dU = exp(s D);  U[cur^1] = U[cur] dU
  double2* dUk = P.dU + (size_t)k * WW;
  #pragma unroll 4
  for (int e = tid; e < WW; e += blockDim.x) dUk[e] = a[e];
  __syncthreads();
  const int cur = st->cur;
  double2* Unew = P.U[cur ^ 1] + (size_t)k * WW;
  if (ok) ok = E::mm(cx, Unew, P.U[cur] + (size_t)k * WW, nullptr, a, ra.col, W, Epi{Unew, 0, Rec{nullptr, nullptr}},
                     none);
  if (tid == 0) atomicAdd(&st->exp_products, (double)s_plan[4] + 1.0);   // the plan's cost, + U dU
  if (!ok && tid == 0) {
    st->error = 2;
    st->done = 1;
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(cx.tmem), "r"((uint32_t)E::TMEM_COLS) : "memory");
  }
}

template <int WP, bool SM>
static cudaError_t oz_exp_launch_wp(const Problem* probs, WorkMap wm, int which, int grid, cudaStream_t s) {
  k_oz_exp<WP, SM><<<grid, 256, ExpProd<WP, SM>::BYTES, s>>>(probs, wm, which);
  return cudaGetLastError();
}

// smem_mats: num_wann 17..32, keep the chain's FP64 matrices in shared memory
cudaError_t oz_exp_launch(int wp, int smem_mats, const Problem* probs, WorkMap wm, int which, int grid,
                          cudaStream_t s) {
  switch (wp) {
    case 8: return oz_exp_launch_wp<8, false>(probs, wm, which, grid, s);
    case 16: return oz_exp_launch_wp<16, false>(probs, wm, which, grid, s);
    case 32:
      return smem_mats ? oz_exp_launch_wp<32, true>(probs, wm, which, grid, s)
                       : oz_exp_launch_wp<32, false>(probs, wm, which, grid, s);
    case 64: return oz_exp_launch_wp<64, false>(probs, wm, which, grid, s);
    default: return oz_exp_launch_wp<128, false>(probs, wm, which, grid, s);
  }
}

template <int WP, bool SM>
static cudaError_t oz_exp_attr_wp() {
  return cudaFuncSetAttribute(k_oz_exp<WP, SM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)ExpProd<WP, SM>::BYTES);
}

cudaError_t oz_exp_set_attributes(int wp, int smem_mats) {
  switch (wp) {
    case 8: return oz_exp_attr_wp<8, false>();
    case 16: return oz_exp_attr_wp<16, false>();
    case 32: return smem_mats ? oz_exp_attr_wp<32, true>() : oz_exp_attr_wp<32, false>();
    case 64: return oz_exp_attr_wp<64, false>();
    default: return oz_exp_attr_wp<128, false>();
  }
}

}  // namespace w90g
