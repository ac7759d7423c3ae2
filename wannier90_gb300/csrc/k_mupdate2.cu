// Tensor-core M update for num_wann <= 32, pipelined: M(k,b) = U(k)^H M0(k,b) U(k+b).
//
// The arithmetic is k_tensor.cu's (real embedding, 7 signed 7-bit FP16 digits per
// operand, the 28 digit pairs of the 7 diagonals accumulated exactly in FP32 TMEM
// columns, exact int64 recombination), so results are bitwise those of k_oz_mupdate;
// only the schedule differs.  One persistent CTA per SM walks the work units
// (group g, 128-row tile) of its share of the groups, with warp-specialised roles
// connected by mbarriers:
//
//   producer warps (4 in step 1, 8 in step 2): per group, the column scales of the
//               shared operand and its 7 digit planes (double-buffered B); per tile, the
//               A operand one K-step (16 real K, all 7 planes, 28 KB) at a time into a ring
//               of stages -- step 1 as one bulk copy per stage from the digit image of the
//               entry overlaps (k_oz_preslice2), step 2 by slicing Z in registers;
//   one warp    MMA issue (one thread): per stage the 28 digit-pair MMAs, a commit that
//               frees the stage, a commit per tile that hands the accumulators over;
//   epilogue warps (16 in step 1, 8 in step 2; 4 or 2 column groups per TMEM lane
//               quarter): TMEM -> registers, exact recombination, FP64 stores (and in
//               step 1 the row scales step 2 will use, by a segmented warp max; in step
//               2 the diagonal statistics of the spread).
//
// While the epilogue drains one tile, the producer fills the stages of the next ones and
// (num_wann <= 16, where two accumulator sets fit the 512 TMEM columns) the MMAs of the
// next tile run.  The K dimension of a tile is ordered per K-step as [Re of 8 complex
// indices, Im of the same 8] (both operands alike), so a producer thread slices each
// complex element once; the order of an exact integer reduction does not change it.
//
// Every wait is bounded (W90G_SPIN_LIMIT tries) and also gives up when another role has
// failed; a failed CTA then waits (W90G_DRAIN_LIMIT) for the MMAs it issued and the bulk
// copies in flight before it frees tensor memory, and reports error 2 for the problem.
#include "oz.cuh"

namespace w90g {

namespace {

constexpr int kDynBudget = 232448 - 5120;                 // opt-in smem minus static use and slack

// Warp roles per step: 16 epilogue warps (4 per TMEM lane quarter) share the exact
// recombination; the producer is split into an A producer, which fills the ring of K-step
// stages, and a B producer, which slices the next group's shared operand into the other B
// buffer meanwhile.  Step 1's A operand arrives by bulk copy (one thread issues it), so its
// B producer gets 3 warps; step 2 slices Z, so its A producer gets 4 warps and B one.
// (21-22 warps: at most 6 per SM sub-partition, so at most 80 registers per thread.)
template <int STEP>
struct Roles {
  static constexpr int EPI = 16;                           // epilogue warps 0 .. EPI-1
  static constexpr int PA = STEP == 1 ? 1 : 4;             // A producer warps EPI ..
  static constexpr int PB = STEP == 1 ? 3 : 1;             // B producer warps EPI + PA ..
  static constexpr int MMA = EPI + PA + PB;                // the MMA-issue warp
  static constexpr int THREADS = (MMA + 1) * 32;
  static constexpr int ET = EPI * 32, PAT = PA * 32, PBT = PB * 32;
  static constexpr int GROUPS = EPI / 4;                   // column groups per lane quarter
  static constexpr int AITEMS = 2 * kTileRows;             // step 2: (row, part) slicing items per stage
  static constexpr int AIPT = (AITEMS + PAT - 1) / PAT;     // ... per A-producer thread
};

constexpr int pow2_cols(int c) { return c <= 32 ? 32 : (c <= 64 ? 64 : (c <= 128 ? 128 : (c <= 256 ? 256 : 512))); }

template <int WP>
struct MU2 {
  static constexpr int kPlanesPerMma = (2 * WP) >= 256 ? 1 : 256 / (2 * WP);   // B planes per MMA (N <= 256)
  static_assert(WP == 8 || WP == 16 || WP == 32, "pipelined M update: num_wann <= 32");
  static constexpr int CW = WP;                    // complex columns (one N chunk)
  static constexpr int KC = 2 * WP;                // real K per tile
  static constexpr int NC = 2 * WP;                // real N
  static constexpr int KSTEPS = KC / 16;           // MMA K-steps per tile
  static constexpr int PLANE = kTileRows * 16 * 2; // one digit plane of one K-step
  static constexpr int STAGE = kS * PLANE;         // 28 KB
  static constexpr int B_PLANE = NC * KC * 2;
  static constexpr int B_BYTES = kS * B_PLANE;
  static constexpr int ACC_COLS = kDiag * NC;
  static constexpr int NACC = (2 * ACC_COLS <= 512) ? 2 : 1;
  static constexpr int TMEM_COLS = pow2_cols(NACC * ACC_COLS);
  static constexpr int NS_RAW = (kDynBudget - 1024 - 2 * B_BYTES) / STAGE;
  static constexpr int NS = NS_RAW > 7 ? 7 : NS_RAW;
  static_assert(NS >= 2, "shared memory for at least two A stages");
  static constexpr size_t BYTES = (size_t)NS * STAGE + 2 * (size_t)B_BYTES + 1024;
};

// element (r, q) of a 128 x 16 K-major stage plane (canonical layout, no swizzle):
// core matrices of 8 rows x 8 K (16 B rows), LBO 128 B along K, SBO 256 B along rows
__device__ __forceinline__ uint32_t stage_off(int r, int q) {
  return (uint32_t)((r >> 3) * 256 + (q >> 3) * 128 + (r & 7) * 16 + (q & 7) * 2);
}

__device__ __forceinline__ void bar_named(int id, int n) {
  asm volatile("bar.sync %0, %1;" :: "r"(id), "r"(n) : "memory");
}

// bounded wait that also stops when another role reported a failure (*bad != 0)
__device__ __forceinline__ bool mbar_wait_role(uint32_t addr, uint32_t parity, volatile int* bad) {
  for (int it = 0; it < W90G_SPIN_LIMIT; ++it) {
    if (mbar_try(addr, parity)) return true;
    if ((it & 63) == 63 && *bad) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" :: "r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(smem_u32(b)) : "memory");
}

// the group's skip predicate, read alike by every role (nothing writes it during the kernel)
__device__ __forceinline__ bool group_active(const Problem& P, int which) {
  const CtrlState* st = P.st;
  return !st->done && !(which == 1 && !st->do_second);
}

template <int WP>
__device__ __forceinline__ int ntiles_of(int B) {
  return (B * WP + kTileRows - 1) / kTileRows;
}

// S = sum_d D_d 2^(7(6-d)) of the 7 diagonal accumulators dd[0], dd[stride], ... (exact
// integers |D_d| < 2^22 held in FP32), exactly.  b_d = bits(D_d + 1.5 * 2^23) = D_d +
// 0x4B400000, and S = 2^21 H + L with H = sum_{d<=3} D_d 2^(7(3-d)), L = sum_{d>=4}
// D_d 2^(7(6-d)): each a sum of widened 32 x 32-bit products with the bias folded into
// one constant.  The same integer as the Horner form (acc << 7) + D_d of k_tensor.cu.
__device__ __forceinline__ long long recombine7_exact(const uint32_t* dd, int stride) {
  long long b[kDiag];
#pragma unroll
  for (int d = 0; d < kDiag; ++d) b[d] = (long long)__float_as_int(__uint_as_float(dd[d * stride]) + 12582912.0f);
  const long long H = b[0] * (1LL << 21) + b[1] * (1LL << 14) + b[2] * 128LL + b[3] - 0x4B400000LL * 2113665LL;
  const long long L = b[4] * (1LL << 14) + b[5] * 128LL + b[6] - 0x4B400000LL * 16513LL;
  return H * (1LL << 21) + L;
}

}  // namespace

// STEP 1: group = k, A = rows of M0(k,b) (digit image), B = conj(U(k)), out Z (tbuf) and
//         the row exponents of step 2 (zexp).  STEP 2: group = k', A = rows of Z(k,b) for
//         the B pairs with nnlist(k,b) = k', B = U(k'), out M and the diagonal statistics.
// ngroups: work items of the map (one per group); grid: persistent, <= ngroups.
template <int WP, int STEP>
__global__ void __launch_bounds__(Roles<STEP>::THREADS, 1)
    k_oz_mupdate2(const Problem* __restrict__ probs, WorkMap wm, int which, int ngroups) {
  using L = MU2<WP>;
  using R = Roles<STEP>;
  constexpr int CW = L::CW, KC = L::KC, NC = L::NC, KSTEPS = L::KSTEPS, NS = L::NS, NACC = L::NACC;
  constexpr int kPlanesPerMma = L::kPlanesPerMma;

  constexpr int kEpiWarps = R::EPI, kMmaWarp = R::MMA, kEpiThreads = R::ET;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;                                 // NS stages
  unsigned char* sB = base + (size_t)NS * L::STAGE;         // 2 B buffers
  __shared__ __align__(8) uint64_t a_full[NS], a_empty[NS];
  __shared__ __align__(8) uint64_t b_full[2], b_empty[2];
  __shared__ __align__(8) uint64_t acc_full[NACC], acc_empty[NACC];
  __shared__ __align__(8) uint64_t drain_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_colexp[2][WP];
  __shared__ volatile int s_bad;
  __shared__ int s_bad_prob;
  __shared__ int s_aflag, s_bflag;
  __shared__ int s_eflag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(&tmem_slot)), "r"((uint32_t)L::TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&a_full[s], STEP == 1 ? 1u : (uint32_t)R::PAT);
      mbar_init(&a_empty[s], 1u);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&b_full[b], STEP == 1 ? (uint32_t)R::PBT : 1u);
      mbar_init(&b_empty[b], 1u + (uint32_t)kEpiThreads);
    }
    for (int a = 0; a < NACC; ++a) {
      mbar_init(&acc_full[a], 1u);
      mbar_init(&acc_empty[a], (uint32_t)kEpiThreads);
    }
    mbar_init(&drain_bar, 1u);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_bad = 0;
    s_bad_prob = -1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  auto fail = [&](int p) {
    if (!s_bad) {
      s_bad_prob = p;
      s_bad = 1;
    }
  };

  if (warp >= kEpiWarps && warp < kEpiWarps + R::PA) {
    // =========================== A producer ===========================
    const int pa = tid - kEpiThreads;
    int sseq = 0;          // stages filled
    uint32_t inflight = 0, inflight_par = 0;   // step 1: slots with a bulk copy issued, and its parity
    // A-producer-wide bounded wait: thread 0 polls, the outcome is shared (uniform branch);
    // in step 1 thread 0 is the whole A producer
    auto await = [&](uint64_t* bar, uint32_t parity, int p) -> bool {
      if (pa == 0) {
        const bool ok = mbar_wait_role(smem_u32(bar), parity, &s_bad);
        if (!ok) fail(p);
        s_aflag = ok ? 0 : 1;
      }
      if (STEP == 1) return s_aflag == 0;
      bar_named(1, R::PAT);
      const bool ok = s_aflag == 0;
      bar_named(1, R::PAT);
      return ok;
    };
    bool ok = STEP == 2 || pa == 0;
    for (int item = blockIdx.x; item < ngroups && ok; item += gridDim.x) {
      int g;
      const int p = locate(wm, item, g);
      const Problem& P = probs[p];
      if (!group_active(P, which)) continue;
      const int W = P.W, B = P.B, WW = W * W;
      const int ntiles = ntiles_of<WP>(B);
      for (int tile = 0; tile < ntiles && ok; ++tile) {
        // step 2: the Z rows this thread slices -- items it = pa + j PAT: tile row it % 128,
        // part it / 128, 8 complex of one K-step (one 16-byte core-matrix row per plane)
        const double2* zrow[R::AIPT];
        int zex[R::AIPT];
        if (STEP == 2) {
#pragma unroll
          for (int j = 0; j < R::AIPT; ++j) {
            const int it = pa + j * R::PAT;
            const int rw = tile * kTileRows + it % kTileRows;
            const int b2 = rw / WP, r2 = rw % WP;
            zrow[j] = nullptr;
            zex[j] = 0;
            if (it < R::AITEMS && b2 < B && r2 < W) {
              const size_t kb = (size_t)P.inv_nnlist[(size_t)g * B + b2];
              zrow[j] = P.tbuf + kb * WW + (size_t)r2 * W;
              zex[j] = P.zexp[kb * W + r2];     // the row's scale, computed by step 1's epilogue
            }
          }
        }
        for (int ks = 0; ks < KSTEPS; ++ks) {
          const int s = sseq % NS;
          const uint32_t use = (uint32_t)(sseq / NS);
          double av[R::AIPT][8];
          if (STEP == 2) {
            // the stage's elements, loaded before the slot is free
#pragma unroll
            for (int j = 0; j < R::AIPT; ++j) {
              const int part = (pa + j * R::PAT) / kTileRows;
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                const int m = ks * 8 + i;
                av[j][i] = (zrow[j] && m < W) ? ((const double*)(zrow[j] + m))[part] : 0.0;
              }
            }
          }
          // (the first use of each stage slot needs no wait)
          if (use > 0 && !await(&a_empty[s], (use & 1) ^ 1, p)) {
            ok = false;
            break;
          }
          inflight &= ~(1u << s);    // the MMA consumed the slot's last copy
          unsigned char* dA = sA + (size_t)s * L::STAGE;
          if (STEP == 1) {
            const unsigned char* src =
                P.m0s + ((((size_t)g * ntiles + tile) * KSTEPS) + ks) * (size_t)L::STAGE;
            asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                         :: "r"(smem_u32(&a_full[s])), "r"((uint32_t)L::STAGE) : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                :: "r"(smem_u32(dA)), "l"(src), "r"((uint32_t)L::STAGE), "r"(smem_u32(&a_full[s]))
                : "memory");
            inflight |= 1u << s;
            inflight_par = (inflight_par & ~(1u << s)) | ((use & 1) << s);
          } else {
            // 128 rows x 8 complex: each item is one part of a row's 8 elements, sliced into
            // all 7 planes (K 0-7 real parts, 8-15 imaginary parts), one 16-byte store each
#pragma unroll
            for (int j = 0; j < R::AIPT; ++j) {
              const int it = pa + j * R::PAT;
              if (it < R::AITEMS) {
                uint32_t w[kS][4];
                pack_digits7(w, av[j], zex[j], false);
                const uint32_t o = stage_off(it % kTileRows, 8 * (it / kTileRows));
#pragma unroll
                for (int t = 0; t < kS; ++t)
                  *(uint4*)(dA + (size_t)t * L::PLANE + o) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
              }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&a_full[s]);
          }
          ++sseq;
        }
      }
    }
    // drain: bulk copies still in flight must land before the CTA frees its shared memory
    if (STEP == 1 && pa == 0)
      for (int s = 0; s < NS; ++s)
        if (inflight & (1u << s)) mbar_drain(smem_u32(&a_full[s]), (inflight_par >> s) & 1);
  } else if (warp >= kEpiWarps + R::PA && warp < kMmaWarp) {
    // =========================== B producer ===========================
    // Step 1 slices conj(U(k)) into the B buffer and also writes the planes of U(k) as step
    // 2 uses them (the same three digit decompositions, Re U, Im U and -Im U, with the two
    // imaginary quadrants exchanged) to the per-k image ub2, with the column exponents
    // (conjugation keeps the moduli).  Step 2 takes its group's B from that image with one
    // bulk copy.
    const int pb = tid - kEpiThreads - R::PAT;
    int gseq = 0;          // groups started
    uint32_t inflight = 0, inflight_par = 0;   // step 2: buffers with a bulk copy issued, and its parity
    auto bwait = [&](uint64_t* bar, uint32_t parity, int p) -> bool {
      if (pb == 0) {
        const bool ok = mbar_wait_role(smem_u32(bar), parity, &s_bad);
        if (!ok) fail(p);
        s_bflag = ok ? 0 : 1;
      }
      bar_named(3, R::PBT);
      const bool ok = s_bflag == 0;
      bar_named(3, R::PBT);
      return ok;
    };
    for (int item = blockIdx.x; item < ngroups; item += gridDim.x) {
      int g;
      const int p = locate(wm, item, g);
      const Problem& P = probs[p];
      if (!group_active(P, which)) continue;
      const int W = P.W, WW = W * W;
      const double2* Ug = P.U[P.st->cur ^ 1] + (size_t)g * WW;
      const int bb = gseq & 1;
      // (the first use of each B buffer needs no wait)
      if (gseq >= 2 && !bwait(&b_empty[bb], ((gseq >> 1) & 1) ^ 1, p)) break;
      unsigned char* dB = sB + (size_t)bb * L::B_BYTES;
      if constexpr (STEP == 2) {
        // column scales and planes from step 1's image of U(k')
        for (int c = pb; c < WP; c += R::PBT) s_colexp[bb][c] = P.ub2_exp[(size_t)g * WP + c];
        bar_named(3, R::PBT);
        inflight &= ~(1u << bb);   // the buffer's previous copy was consumed (b_empty)
        if (pb == 0) {
          const unsigned char* src = P.ub2 + (size_t)g * L::B_BYTES;
          asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                       :: "r"(smem_u32(&b_full[bb])), "r"((uint32_t)L::B_BYTES) : "memory");
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
              :: "r"(smem_u32(dB)), "l"(src), "r"((uint32_t)L::B_BYTES), "r"(smem_u32(&b_full[bb]))
              : "memory");
          inflight |= 1u << bb;
          inflight_par = (inflight_par & ~(1u << bb)) | ((((uint32_t)gseq >> 1) & 1u) << bb);
        }
        ++gseq;
      } else {
      // column scales: one column per thread, 8 independent loads per round
      for (int c = pb; c < WP; c += R::PBT) {
        unsigned long long mx = 0ull;
        if (c < W)
          for (int m0 = 0; m0 < W; m0 += 8) {
            double2 v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = (m0 + i < W) ? Ug[(size_t)c * W + m0 + i] : make_double2(0.0, 0.0);
#pragma unroll
            for (int i = 0; i < 8; ++i) mx = max(mx, max(abs_bits(v[i].x), abs_bits(v[i].y)));
          }
        s_colexp[bb][c] = exp_above_bits(mx);
        if (P.ub2_exp) P.ub2_exp[(size_t)g * WP + c] = exp_above_bits(mx);
      }
      bar_named(3, R::PBT);
      unsigned char* gB = P.ub2 ? P.ub2 + (size_t)g * L::B_BYTES : nullptr;   // step 2's image of U(k)
      // B^T planes: each complex U(m, c) gives the four real entries of the embedding
      // [[B_r, B_i], [-B_i, B_r]]; B_r, B_i and -B_i are sliced once each.  A thread takes
      // one part of 8 consecutive m of column c (contiguous in memory; their K positions
      // form one 16-byte core-matrix row) and stores each plane's row with 16-byte stores:
      // B_r to (N re, K re) and (N im, K im); B_i to (N im, K re), -B_i to (N re, K im).
      for (int idx = pb; idx < WP * (WP / 8) * 2; idx += R::PBT) {
        const int cc = idx % WP, g8 = (idx / WP) % (WP / 8), part = idx / (WP * (WP / 8));
        const int ec = s_colexp[bb][cc];
        double v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int mm = g8 * 8 + i;
          v[i] = 0.0;
          if (cc < W && mm < W) {
            const double2 u = Ug[(size_t)cc * W + mm];
            v[i] = part == 0 ? u.x : -u.y;     // step 1: B = conj(U)
          }
        }
        uint32_t w[kS][4];
        pack_digits7(w, v, ec, false);
        const int k_re = g8 * 16, k_im = k_re + 8;   // K positions of Re / Im of m = 8 g8 ..
        if (part == 0) {
          const uint32_t o_rr = kmaj_off(cc, k_re, KC), o_ii = kmaj_off(CW + cc, k_im, KC);
#pragma unroll
          for (int t = 0; t < kS; ++t) {
            const uint4 q = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
            unsigned char* pl = dB + (size_t)t * L::B_PLANE;
            *(uint4*)(pl + o_rr) = q;   // (K re, N re) = B_r
            *(uint4*)(pl + o_ii) = q;   // (K im, N im) = B_r
            if (gB) {
              *(uint4*)(gB + (size_t)t * L::B_PLANE + o_rr) = q;
              *(uint4*)(gB + (size_t)t * L::B_PLANE + o_ii) = q;
            }
          }
        } else {
          // B_i = -Im U (step 1) to (N im, K re) -- for step 2 (B_i = Im U) the same digits
          // go to (N re, K im) -- and -B_i = Im U to (N re, K im), for step 2 to (N im, K re)
          const uint32_t o_ir = kmaj_off(CW + cc, k_re, KC), o_ri = kmaj_off(cc, k_im, KC);
#pragma unroll
          for (int t = 0; t < kS; ++t) {
            const uint4 q = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
            *(uint4*)(dB + (size_t)t * L::B_PLANE + o_ir) = q;
            if (gB) *(uint4*)(gB + (size_t)t * L::B_PLANE + o_ri) = q;
          }
          pack_digits7(w, v, ec, true);
#pragma unroll
          for (int t = 0; t < kS; ++t) {   // the digits of the negated values
            const uint4 q = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
            *(uint4*)(dB + (size_t)t * L::B_PLANE + o_ri) = q;
            if (gB) *(uint4*)(gB + (size_t)t * L::B_PLANE + o_ir) = q;
          }
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&b_full[bb]);
      ++gseq;
      }
    }
    // drain (step 2): bulk copies still in flight must land before the CTA frees its memory
    if (STEP == 2 && pb == 0)
      for (int b = 0; b < 2; ++b)
        if (inflight & (1u << b)) mbar_drain(smem_u32(&b_full[b]), (inflight_par >> b) & 1);
  } else if (warp == kMmaWarp) {
    // =========================== MMA issue ===========================
    if (lane == 0) {
      int gseq = 0, sseq = 0, useq = 0;
      bool issued = false, ok = true;
      for (int item = blockIdx.x; item < ngroups && ok; item += gridDim.x) {
        int g;
        const int p = locate(wm, item, g);
        const Problem& P = probs[p];
        if (!group_active(P, which)) continue;
        const int ntiles = ntiles_of<WP>(P.B);
        const int bb = gseq & 1;
        if (!mbar_wait_role(smem_u32(&b_full[bb]), (gseq >> 1) & 1, &s_bad)) {
          fail(p);
          break;
        }
        const uint32_t b0 = smem_u32(sB + (size_t)bb * L::B_BYTES);
        for (int tile = 0; tile < ntiles && ok; ++tile) {
          const int a = useq % NACC;
          const uint32_t ause = (uint32_t)(useq / NACC);
          // (the first use of each accumulator set needs no wait)
          if (ause > 0 && !mbar_wait_role(smem_u32(&acc_empty[a]), (ause & 1) ^ 1, &s_bad)) {
            fail(p);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t acc = tmem + (uint32_t)(a * L::ACC_COLS);
          for (int ks = 0; ks < KSTEPS; ++ks) {
            const int s = sseq % NS;
            if (!mbar_wait_role(smem_u32(&a_full[s]), (uint32_t)(sseq / NS) & 1, &s_bad)) {
              fail(p);
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // descriptors: the base descriptor plus the byte offset / 16 in the address field
            // (shared-memory addresses stay below 2^18, so the field holds it)
            const uint64_t da = smem_desc(smem_u32(sA + (size_t)s * L::STAGE), 128, 256);
            const uint64_t db = smem_desc(b0 + ks * 256, 128, (KC / 8) * 128);
            // The B planes follow one another as consecutive row groups of one K-major
            // operand, and diagonal d's accumulator columns follow d - 1's: digit plane t
            // of A against planes u0 .. u0 + n - 1 of B is one MMA with N = n NC, writing
            // diagonals t + u0 .. at once (N <= 256).  The integer sums are exact, so the
            // grouping does not change them.
#pragma unroll
            for (int t = 0; t < kS; ++t) {
              const uint64_t ad = da + (uint64_t)((t * L::PLANE) >> 4);
#pragma unroll
              for (int u0 = 0; u0 + t <= kS - 1; u0 += kPlanesPerMma) {
                const int n = (kS - t - u0) < kPlanesPerMma ? (kS - t - u0) : kPlanesPerMma;
                const uint64_t bd = db + (uint64_t)((u0 * L::B_PLANE) >> 4);
                // the first write of every diagonal in this tile: plane 0 of A, K-step 0
                const uint32_t accf = (ks == 0 && t == 0) ? 0u : 1u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    :: "r"(acc + (uint32_t)((t + u0) * NC)), "l"(ad), "l"(bd), "r"(idesc_f16(n * NC)), "r"(accf)
                    : "memory");
              }
            }
            issued = true;
            mma_commit(&a_empty[s]);          // the stage is free once these MMAs completed
            ++sseq;
          }
          if (!ok) break;
          mma_commit(&acc_full[a]);           // the tile's accumulators are complete
          if (tile == ntiles - 1) mma_commit(&b_empty[bb]);
          ++useq;
        }
        ++gseq;
      }
      // drain: no MMA may still write tensor memory when it is freed
      if (issued) {
        mma_commit(&drain_bar);
        mbar_drain(smem_u32(&drain_bar), 0);
      }
    }
  } else {
    // =========================== epilogue ===========================
    const int wq = warp & 3, cg = warp >> 2;            // TMEM lane quarter, column group
    const int r = wq * 32 + lane;                       // tile row = TMEM lane
    const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
    constexpr int CPG = CW / R::GROUPS;                 // complex columns per warp
    const int jbeg = cg * CPG;
    int gseq = 0, useq = 0;
    bool ok = true;
    for (int item = blockIdx.x; item < ngroups && ok; item += gridDim.x) {
      int g;
      const int p = locate(wm, item, g);
      const Problem& P = probs[p];
      if (!group_active(P, which)) continue;
      const int W = P.W, B = P.B, WW = W * W;
      const int cur = P.st->cur;
      const int ntiles = ntiles_of<WP>(B);
      const int bb = gseq & 1;
      for (int tile = 0; tile < ntiles && ok; ++tile) {
        const int a = useq % NACC;
        const uint32_t ause = (uint32_t)(useq / NACC);
        // the row's scale and output block, fetched before the accumulators are ready
        const int row = tile * kTileRows + r;
        const int bi = row / WP, rr = row % WP;
        const bool valid = (bi < B) && (rr < W);
        int erow = 0, kb_out = 0;
        if (STEP == 1) {
          erow = P.m0s_exp[((size_t)g * ntiles + tile) * kTileRows + r];
        } else if (bi < B) {
          kb_out = P.inv_nnlist[(size_t)g * B + bi];
          if (valid) erow = P.zexp[(size_t)kb_out * W + rr];
        }
        const size_t kb_in = (size_t)g * B + bi;    // step 1: block (k, b) of this row
        // one epilogue thread waits for the accumulators; the others wait at the epilogue
        // group's named barrier (issuing nothing) and read the outcome
        if (tid == 0) {
          const bool okw = mbar_wait_role(smem_u32(&acc_full[a]), ause & 1, &s_bad);
          if (!okw) fail(p);
          s_eflag = okw ? 0 : 1;
        }
        bar_named(2, kEpiThreads);
        const bool okw = s_eflag == 0;
        bar_named(2, kEpiThreads);
        if (!okw) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        int ecol[CPG];
#pragma unroll
        for (int j = 0; j < CPG; ++j) ecol[j] = s_colexp[bb][jbeg + j];
        if (tile == ntiles - 1) mbar_arrive(&b_empty[bb]);   // colexp read: B may be replaced
        const uint32_t acc = tmem + (uint32_t)(a * L::ACC_COLS);
        double dre = 0.0, dim = 0.0;
        bool has_diag = false;
#pragma unroll 1
        for (int j0 = jbeg; j0 < jbeg + CPG; j0 += 2) {
          uint32_t q[kDiag][2], s2[kDiag][2];
#pragma unroll
          for (int d = 0; d < kDiag; ++d) {
            const uint32_t ta = acc + lane_base + (uint32_t)(d * NC + j0);
            const uint32_t tb = acc + lane_base + (uint32_t)(d * NC + CW + j0);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];"
                         : "=r"(q[d][0]), "=r"(q[d][1]) : "r"(ta));
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];"
                         : "=r"(s2[d][0]), "=r"(s2[d][1]) : "r"(tb));
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int c = j0 + j;   // complex output column
            const int e = erow + ecol[c - jbeg];
            const double re = int64_scaled_to_double(recombine7_exact(&q[0][j], 2), e - 56);
            const double im = int64_scaled_to_double(recombine7_exact(&s2[0][j], 2), e - 56);
            if (STEP == 1) {
              // step 2's row scale of row c of Z(k,b): the largest |re|, |im| over this
              // block's rows rr, i.e. over its WP lanes (segmented max; zero rows add 0).
              // Only the exponent field is used: the max of the high words, and whether
              // any low word is set (a subnormal maximum).
              const unsigned long long ab = valid ? max(abs_bits(re), abs_bits(im)) : 0ull;
              uint32_t hi = (uint32_t)(ab >> 32), lo = (uint32_t)ab;
#pragma unroll
              for (int o = 1; o < WP && o < 32; o <<= 1) {
                hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
                lo |= __shfl_xor_sync(0xffffffffu, lo, o);
              }
              if (valid && c < W) P.tbuf[kb_in * WW + (size_t)c * W + rr] = make_double2(re, im);
              if (rr == 0 && bi < B && c < W)
                P.zexp[kb_in * W + c] = exp_above_bits(((unsigned long long)hi << 32) | (lo ? 1ull : 0ull));
            } else if (valid && c < W) {
              P.M[cur ^ 1][(size_t)kb_out * WW + (size_t)c * W + rr] = make_double2(re, im);
              if (c == rr) {
                dre = re;
                dim = im;
                has_diag = true;
              }
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(&acc_empty[a]);
        if (STEP == 2 && has_diag) {
          P.diag_ln[(size_t)kb_out * W + rr] = guided_ln(P, (size_t)kb_out * W + rr, make_double2(dre, dim));
          P.diag_abs2[(size_t)kb_out * W + rr] = dre * dre + dim * dim;
        }
        ++useq;
      }
      ++gseq;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaWarp) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(tmem), "r"((uint32_t)L::TMEM_COLS) : "memory");
  }
  if (tid == 0 && s_bad && s_bad_prob >= 0) {
    CtrlState* st = probs[s_bad_prob].st;
    st->error = 2;
    st->done = 1;
  }
}

// The digit image of step 1's A operand for the pipelined kernel: per (k, tile, K-step)
// the 7 planes of the 128 x 16 stage, exactly as the producer would slice M0, plus the
// tiles' row exponents.  One CTA (256 threads) per k.
template <int WP>
__global__ void __launch_bounds__(256) k_oz_preslice2(const Problem* __restrict__ probs, WorkMap wm) {
  using L = MU2<WP>;
  constexpr int KSTEPS = L::KSTEPS;
  __shared__ int s_rowexp[kTileRows];
  int g;
  const int p = locate(wm, blockIdx.x, g);
  const Problem& P = probs[p];
  if (!P.m0s) return;
  const int W = P.W, B = P.B, WW = W * W;
  const int ntiles = ntiles_of<WP>(B);
  const int tid = threadIdx.x;
  for (int tile = 0; tile < ntiles; ++tile) {
    // row scales over the full row (2 threads per row)
    {
      const int r = tid >> 1, halfr = tid & 1;
      const int row = tile * kTileRows + r;
      const int bi = row / WP, rr = row % WP;
      unsigned long long mx = 0ull;
      if (bi < B && rr < W)
        for (int m = halfr; m < W; m += 2) {
          const double2 a = P.M0[((size_t)g * B + bi) * WW + (size_t)rr * W + m];
          mx = max(mx, max(abs_bits(a.x), abs_bits(a.y)));
        }
      mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mx, 1));
      if (halfr == 0) s_rowexp[r] = exp_above_bits(mx);
    }
    __syncthreads();
    if (tid < kTileRows) P.m0s_exp[((size_t)g * ntiles + tile) * kTileRows + tid] = s_rowexp[tid];
    for (int ks = 0; ks < KSTEPS; ++ks) {
      unsigned char* dst = P.m0s + (((size_t)g * ntiles + tile) * KSTEPS + ks) * (size_t)L::STAGE;
      for (int e = tid; e < kTileRows * 8; e += blockDim.x) {
        const int r = e >> 3, l = e & 7;
        const int row = tile * kTileRows + r;
        const int bi = row / WP, rr = row % WP;
        const int m = ks * 8 + l;
        double2 a = make_double2(0.0, 0.0);
        if (bi < B && rr < W && m < W) a = P.M0[((size_t)g * B + bi) * WW + (size_t)rr * W + m];
        int xr[kS], xi[kS];
        digits7(scaled_int(a.x, s_rowexp[r]), xr);
        digits7(scaled_int(a.y, s_rowexp[r]), xi);
        const uint32_t o = stage_off(r, l);
#pragma unroll
        for (int t = 0; t < kS; ++t) {
          *(uint16_t*)(dst + (size_t)t * L::PLANE + o) = int_to_f16(xr[t]);
          *(uint16_t*)(dst + (size_t)t * L::PLANE + o + 128) = int_to_f16(xi[t]);
        }
      }
    }
    __syncthreads();
  }
}

// ---- host side ----------------------------------------------------------------------
namespace {

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || n <= 0)
      n = 148;
  }
  return n;
}

template <int WP>
cudaError_t launch2_wp(int step, const Problem* probs, WorkMap wm, int which, int ngroups, cudaStream_t s) {
  const int grid = ngroups < sm_count() ? ngroups : sm_count();
  if (grid <= 0) return cudaSuccess;
  const size_t sm = MU2<WP>::BYTES;
  if (step == 1) k_oz_mupdate2<WP, 1><<<grid, Roles<1>::THREADS, sm, s>>>(probs, wm, which, ngroups);
  else k_oz_mupdate2<WP, 2><<<grid, Roles<2>::THREADS, sm, s>>>(probs, wm, which, ngroups);
  return cudaGetLastError();
}

template <int WP>
cudaError_t attr2_wp() {
  const int sm = (int)MU2<WP>::BYTES;
  cudaError_t e = cudaFuncSetAttribute(k_oz_mupdate2<WP, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_oz_mupdate2<WP, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
}

}  // namespace

// pipelined M update (num_wann <= 32): step 1 or 2 over the ngroups work items of wm
cudaError_t oz2_launch(int wp, int step, const Problem* probs, WorkMap wm, int which, int ngroups,
                       cudaStream_t s) {
  switch (wp) {
    case 8: return launch2_wp<8>(step, probs, wm, which, ngroups, s);
    case 16: return launch2_wp<16>(step, probs, wm, which, ngroups, s);
    case 32: return launch2_wp<32>(step, probs, wm, which, ngroups, s);
    default: return cudaErrorInvalidValue;
  }
}

// bytes of step 2's per-k B image and its column exponents
void oz2_ub2_bytes(int wp, int K, size_t* data, size_t* exps) {
  const size_t b_bytes = (size_t)kS * (2 * wp) * (2 * wp) * 2;
  *data = (size_t)K * b_bytes;
  *exps = (size_t)K * wp * 4;
}

cudaError_t oz2_set_attributes(int wp) {
  switch (wp) {
    case 8: return attr2_wp<8>();
    case 16: return attr2_wp<16>();
    case 32: return attr2_wp<32>();
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t oz2_preslice_launch(int wp, const Problem* probs, WorkMap wm, int grid, cudaStream_t s) {
  switch (wp) {
    case 8: k_oz_preslice2<8><<<grid, 256, 0, s>>>(probs, wm); break;
    case 16: k_oz_preslice2<16><<<grid, 256, 0, s>>>(probs, wm); break;
    case 32: k_oz_preslice2<32><<<grid, 256, 0, s>>>(probs, wm); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace w90g
