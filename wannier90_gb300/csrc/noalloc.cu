// Loewdin projection that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they project --
// for example a DFT code that has handed all of the GPU's memory to its own pool
// allocator, or a code that projects from inside a region where a device allocation is
// not permitted or would stall other streams.  They pass their own M and U buffers; the
// few bytes of descriptor and the per-block statistics the kernels write live in one
// file-scope device array instead of a cudaMalloc'd arena.
//
// Limits: num_wann <= 32, num_kpts <= 4096, num_kpts * nntot <= 8192, every nnkp entry in
// 1..num_kpts (anything else returns 5 before the GPU is touched).  The array holds
// about 4.2 MB and stays allocated on every GPU that loads the library until the process
// exits.  All calls share it: two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on it.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/wannier90_gb300.h"
#include "w90g.cuh"

namespace w90g {

__global__ void k_lowdin(const Problem* probs, WorkMap wm, int* status);
__global__ void k_m_update(const Problem* probs, WorkMap wm, int mode, int which);

namespace {

constexpr int kNaMaxW = 32;
constexpr int kNaMaxK = 4096;
constexpr int kNaMaxKB = 8192;
constexpr int kNaMaxDev = 64;

struct NoAllocScratch {
  Problem prob;                        // descriptor the kernels read
  CtrlState st;                        // kernels read st.cur (must be 0)
  int offs_k[2];
  int offs_kb[2];
  int status[kNaMaxK];                 // per-k result of k_lowdin
  int nnlist[kNaMaxKB];                // [k][b], 0-based
  int nnkp_raw[kNaMaxKB];              // caller's [b][k], 1-based
  double diag_ln[kNaMaxKB * kNaMaxW];  // statistics written by k_m_update's epilogue
  double diag_abs2[kNaMaxKB * kNaMaxW];
  double offd[kNaMaxKB];
};

// The scratch array.  In host code this name is a host-side stand-in, not a device
// address: host code must use the address obtained from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_setup_mu;
NoAllocScratch* g_scratch_addr[kNaMaxDev] = {nullptr};

// nnkp (1-based, [b][k]) -> nnlist (0-based, [k][b]) inside the scratch array
__global__ void k_noalloc_nnlist(int K, int B) {
  NoAllocScratch* s = reinterpret_cast<NoAllocScratch*>(g_noalloc_scratch);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K * B; i += gridDim.x * blockDim.x) {
    const int k = i / B, b = i % B;
    s->nnlist[i] = s->nnkp_raw[b * K + k] - 1;
  }
}

// On every call, with the device current: resolve the scratch address (no allocation
// involved) and, when it differs from the one this device had before -- the first call,
// or a new primary context after cudaDeviceReset -- raise the dynamic shared-memory limit
// of the two kernels again.
int setup_device(int dev, NoAllocScratch** out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (dev < 0 || dev >= kNaMaxDev) return 1;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return 1;
  if (g_scratch_addr[dev] != p) {
    const int smem = 4 * kNaMaxW * kNaMaxW * 16;
    if (cudaFuncSetAttribute(k_lowdin, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
      return 1;
    if (cudaFuncSetAttribute(k_m_update, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
      return 1;
    g_scratch_addr[dev] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_scratch_addr[dev];
  return 0;
}

}  // namespace
}  // namespace w90g

extern "C" int w90g_project_overlap_noalloc(int num_wann, int num_kpts, int nntot, const int* nnkp,
                                            double* d_m_matrix, double* d_u_matrix, void* cuda_stream) {
  using namespace w90g;
  if (num_wann < 1 || num_wann > kNaMaxW || num_kpts < 1 || num_kpts > kNaMaxK || nntot < 1 ||
      nntot > 12 || (long long)num_kpts * nntot > kNaMaxKB || !nnkp || !d_m_matrix || !d_u_matrix)
    return 5;   // sizes beyond the scratch array, or missing buffers
  // the table is a gather index on the GPU: every entry must name a k-point (1-based)
  for (long long i = 0; i < (long long)num_kpts * nntot; ++i)
    if (nnkp[i] < 1 || nnkp[i] > num_kpts) return 5;
  // an error left pending by earlier work of the caller is not cleared here: it is
  // reported as a failure of this call and stays pending for the caller to read
  if (cudaPeekAtLastError() != cudaSuccess) return 1;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  NoAllocScratch* s = nullptr;
  if (setup_device(dev, &s)) return 1;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  const int W = num_wann, K = num_kpts, B = nntot;

  // descriptor and controller state: every field the kernels read is written here, and
  // the state starts at zero (cur = 0) on every call
  Problem P;
  std::memset(&P, 0, sizeof(P));
  P.W = W;
  P.K = K;
  P.B = B;
  P.M[0] = P.M[1] = reinterpret_cast<double2*>(d_m_matrix);
  P.U[0] = P.U[1] = reinterpret_cast<double2*>(d_u_matrix);
  P.nnlist = s->nnlist;
  P.diag_ln = s->diag_ln;
  P.diag_abs2 = s->diag_abs2;
  P.offd = s->offd;
  P.st = &s->st;
  CtrlState cs;
  std::memset(&cs, 0, sizeof(cs));
  const int offs_k[2] = {0, K};
  const int offs_kb[2] = {0, K * B};
  if (cudaMemcpyAsync(&s->prob, &P, sizeof(P), cudaMemcpyHostToDevice, st) != cudaSuccess) return 1;
  if (cudaMemcpyAsync(&s->st, &cs, sizeof(cs), cudaMemcpyHostToDevice, st) != cudaSuccess) return 1;
  if (cudaMemcpyAsync(s->offs_k, offs_k, sizeof(offs_k), cudaMemcpyHostToDevice, st) != cudaSuccess) return 1;
  if (cudaMemcpyAsync(s->offs_kb, offs_kb, sizeof(offs_kb), cudaMemcpyHostToDevice, st) != cudaSuccess) return 1;
  if (cudaMemcpyAsync(s->nnkp_raw, nnkp, sizeof(int) * K * B, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return 1;
  k_noalloc_nnlist<<<(K * B + 255) / 256, 256, 0, st>>>(K, B);
  const size_t smem = (size_t)4 * W * W * 16;
  const WorkMap wmk{s->offs_k, 1};
  const WorkMap wmkb{s->offs_kb, 1};
  k_lowdin<<<K, 256, smem, st>>>(&s->prob, wmk, s->status);
  k_m_update<<<K * B, 256, smem, st>>>(&s->prob, wmkb, 1, 0);
  if (cudaGetLastError() != cudaSuccess) return 1;
  // per-k status: rank-deficient A(k) or an unconverged eigensolver is an error
  int status[kNaMaxK];
  if (cudaMemcpyAsync(status, s->status, sizeof(int) * K, cudaMemcpyDeviceToHost, st) != cudaSuccess) return 1;
  if (cudaStreamSynchronize(st) != cudaSuccess) return 1;
  for (int k = 0; k < K; ++k)
    if (status[k] != 0) return 1;
  return 0;
}
