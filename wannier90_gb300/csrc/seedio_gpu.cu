// .mmn parsed on the GPU, straight into the device-resident overlaps the engine solves on.
//
// The text image is read into pinned host memory and copied to the device; there:
//   1. k_seed_count:   newlines per 4 KB chunk;
//   2. k_seed_scan:    exclusive scan of the chunk counts (one CTA);
//   3. k_seed_starts:  start offset of every record; k_seed_blank flags blank records;
//   4. k_mmn_heads:    the block headers (k, k2, G) -> neighbour slot nn, as overlap_read
//                      matches them against nnlist / nncell (src/overlap.F90:268-300);
//   5. k_mmn_values:   one thread per value record, two numbers each, written to
//                      m(:, :, nn, k).
// Numbers are converted with Clinger's fast path: a decimal with at most 19 significant
// digits whose integer mantissa is below 2^53 and whose power of ten is within 10^+-22 is
// exactly one IEEE multiplication or division of two exact doubles, hence correctly
// rounded -- the same double a correctly rounded reader (std::from_chars) returns.  Files
// outside that fast path (more digits, far exponents), with blank records, two blocks for
// one neighbour slot, or anything malformed are handed to the host reader, so the result
// never depends on which path ran.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "seedio.h"

namespace w90g {

namespace {

constexpr int kChunk = 4096;

__constant__ double c_pow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                   1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

__device__ __forceinline__ bool is_sep(char c) { return c == ' ' || c == '\t' || c == ',' || c == '\r'; }

// next item of [p, e): returns its start, sets q past it; nullptr when none is left
__device__ __forceinline__ const char* next_item(const char* p, const char* e, const char*& q) {
  while (p < e && is_sep(*p)) ++p;
  if (p >= e) return nullptr;
  q = p;
  while (q < e && !is_sep(*q)) ++q;
  return p;
}

__device__ bool parse_int(const char* b, const char* e, int& v) {
  bool neg = false;
  if (b < e && (*b == '+' || *b == '-')) neg = (*b++ == '-');
  if (b >= e || e - b > 9) return false;
  int x = 0;
  for (; b < e; ++b) {
    if (*b < '0' || *b > '9') return false;
    x = x * 10 + (*b - '0');
  }
  v = neg ? -x : x;
  return true;
}

// Clinger fast path; false = not representable by it (the host reader takes the file)
__device__ bool parse_double(const char* b, const char* e, double& v) {
  bool neg = false;
  if (b < e && (*b == '+' || *b == '-')) neg = (*b++ == '-');
  unsigned long long mant = 0;
  int ndig = 0, dexp = 0;
  bool digits = false, point = false;
  for (; b < e; ++b) {
    const char c = *b;
    if (c >= '0' && c <= '9') {
      digits = true;
      if (mant == 0 && c == '0') {
        if (point) --dexp;   // leading zeros after the point only shift the exponent
        continue;
      }
      if (ndig >= 19) return false;
      mant = mant * 10 + (unsigned long long)(c - '0');
      ++ndig;
      if (point) --dexp;
    } else if (c == '.' && !point) {
      point = true;
    } else {
      break;
    }
  }
  if (!digits) return false;
  if (b < e) {
    const char c = *b;
    if (!(c == 'e' || c == 'E' || c == 'd' || c == 'D')) return false;
    ++b;
    int x = 0;
    if (!parse_int(b, e, x)) return false;
    dexp += x;
  }
  if (mant == 0) {
    v = neg ? -0.0 : 0.0;
    return true;
  }
  if (mant > (1ull << 53) || dexp < -22 || dexp > 22) return false;
  const double m = (double)mant;   // exact
  const double r = dexp >= 0 ? m * c_pow10[dexp] : m / c_pow10[-dexp];
  v = neg ? -r : r;
  return true;
}

__global__ void k_seed_count(const char* __restrict__ txt, size_t n, int* __restrict__ counts) {
  const size_t c = blockIdx.x;
  const size_t lo = c * kChunk, hi = min(n, lo + kChunk);
  int cnt = 0;
  for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) cnt += (txt[i] == '\n');
  // block sum (blockDim 256)
  __shared__ int s[256];
  s[threadIdx.x] = cnt;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[c] = s[0];
}

// exclusive scan of counts[0..nc) in place, total in *total; one CTA of 1024 threads
__global__ void k_seed_scan(int* counts, int nc, int* total) {
  __shared__ int s[1024];
  const int t = threadIdx.x;
  const int per = (nc + 1023) / 1024;
  const int lo = t * per, hi = min(nc, lo + per);
  int sum = 0;
  for (int i = lo; i < hi; ++i) sum += counts[i];
  s[t] = sum;
  __syncthreads();
  for (int w = 1; w < 1024; w <<= 1) {
    const int v = (t >= w) ? s[t - w] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  int run = s[t] - sum;
  for (int i = lo; i < hi; ++i) {
    const int c = counts[i];
    counts[i] = run;
    run += c;
  }
  if (t == 1023) *total = s[1023];
}

// starts[0] = 0, starts[r+1] = position after the r-th newline (0-based r).  One warp per
// 4 KB chunk: lane l scans bytes [l*128, (l+1)*128) of it (eight 16-byte loads), an
// exclusive shuffle scan of the lanes' newline counts gives each lane its first record.
__global__ void k_seed_starts(const char* __restrict__ txt, size_t n, const int* __restrict__ offs,
                              long long* __restrict__ starts) {
  constexpr int kLane = kChunk / 32;
  const size_t c = blockIdx.x;
  const int lane = threadIdx.x;
  const size_t lo = c * kChunk + (size_t)lane * kLane;
  const size_t hi = min(n, lo + kLane);
  // the text buffer is 16-byte aligned (cudaMallocAsync) and chunk / lane spans are
  // multiples of 16, so whole 16-byte vectors can be loaded up to the last full one
  int cnt = 0;
  if (lo < hi) {
    if (hi - lo == (size_t)kLane) {
      const uint4* v = reinterpret_cast<const uint4*>(txt + lo);
#pragma unroll
      for (int q = 0; q < kLane / 16; ++q) {
        const uint4 w = v[q];
        const unsigned int u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int h = 0; h < 4; ++h)
#pragma unroll
          for (int bt = 0; bt < 4; ++bt) cnt += (((u[h] >> (8 * bt)) & 0xffu) == (unsigned)'\n');
      }
    } else {
      for (size_t i = lo; i < hi; ++i) cnt += (txt[i] == '\n');
    }
  }
  int inc = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  int r = offs[c] + inc - cnt;
  for (size_t i = lo; i < hi; ++i)
    if (txt[i] == '\n') starts[++r] = (long long)i + 1;
  if (c == 0 && lane == 0) starts[0] = 0;
}

// blank-record check over records [first, nrec)
__global__ void k_seed_blank(const char* __restrict__ txt, const long long* __restrict__ starts, long long nrec,
                             long long first, int* flags) {
  for (long long r = first + blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nrec;
       r += (long long)gridDim.x * blockDim.x) {
    const char* b = txt + starts[r];
    const char* e = txt + starts[r + 1] - 1;   // the newline
    bool bl = true;
    for (const char* p = b; p < e && bl; ++p) bl = is_sep(*p);
    if (bl) atomicOr(flags, 1);
  }
}

__global__ void k_mmn_heads(const char* __restrict__ txt, const long long* __restrict__ starts, int nk, int nntot,
                            long long per, const int* __restrict__ nnlist, const int* __restrict__ nncell,
                            int* __restrict__ dest, int* flags) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= (long long)nk * nntot) return;
  const long long r = 2 + j * per;
  const char* p = txt + starts[r];
  const char* e = txt + starts[r + 1] - 1;
  int v[5];
  for (int i = 0; i < 5; ++i) {
    const char* q;
    const char* b = next_item(p, e, q);
    if (!b || !parse_int(b, q, v[i])) {
      atomicOr(flags, 2);
      return;
    }
    p = q;
  }
  const int k = v[0] - 1, k2 = v[1] - 1;
  if (k < 0 || k >= nk) {
    atomicOr(flags, 2);
    return;
  }
  int nn = -1, hits = 0;
  for (int i = 0; i < nntot; ++i) {
    const long long o = (long long)k * nntot + i;
    if (nnlist[o] == k2 && nncell[3 * o] == v[2] && nncell[3 * o + 1] == v[3] && nncell[3 * o + 2] == v[4]) {
      ++hits;
      nn = i;
    }
  }
  if (hits != 1) {
    atomicOr(flags, 2);
    return;
  }
  dest[j] = k * nntot + nn;
}

__global__ void k_mmn_values(const char* __restrict__ txt, const long long* __restrict__ starts, long long nblk,
                             long long per, long long nn2, const int* __restrict__ dest, double2* __restrict__ m,
                             int* flags) {
  const long long total = nblk * (per - 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long j = t / (per - 1), i = t % (per - 1);
    const long long r = 2 + j * per + 1 + i;
    const char* p = txt + starts[r];
    const char* e = txt + starts[r + 1] - 1;
    double x[2];
    bool ok = true;
    for (int c = 0; c < 2 && ok; ++c) {
      const char* q;
      const char* b = next_item(p, e, q);
      ok = b && parse_double(b, q, x[c]);
      p = q;
    }
    if (!ok) {
      atomicOr(flags, 4);
      continue;
    }
    m[(long long)dest[j] * nn2 + i] = make_double2(x[0], x[1]);
  }
}

}  // namespace

#define SEED_CHECK(call)                                                          \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                   \
      rc = (e_ == cudaErrorMemoryAllocation) ? 2 : 1;                             \
      goto done;                                                                  \
    }                                                                             \
  } while (0)

int read_mmn_device(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell, double* d_m,
                    cudaStream_t st, int* used_gpu, long long* launches, double* timing3, std::string& err) {
  *used_gpu = 0;
  *launches = 0;
  int rc = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  if (timing3) {
    timing3[0] = timing3[1] = timing3[2] = 0.0;
    for (auto& e : ev) cudaEventCreate(&e);
  }
  char* h_txt = nullptr;
  char* d_txt = nullptr;
  int *d_counts = nullptr, *d_flags = nullptr, *d_total = nullptr, *d_dest = nullptr, *d_nnl = nullptr,
      *d_ncell = nullptr;
  long long* d_starts = nullptr;
  size_t n = 0;
  int h_flags = 0, h_total = 0;
  const long long nblk = (long long)nk * nntot, per = 1 + (long long)nb * nb;
  const long long nrec_needed = 2 + nblk * per;
  std::vector<int> dest;
  bool fallback = false;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) {
      err = std::string("Error: Problem opening input file ") + path;
      return 6;
    }
    std::fseek(f, 0, SEEK_END);
    const long len = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (len <= 0) {
      std::fclose(f);
      err = std::string("Error: Problem reading input file ") + path;
      return 6;
    }
    n = (size_t)len;
    // one extra byte: a final newline when the file has none
    if (cudaMallocHost(&h_txt, n + 1) != cudaSuccess) {
      std::fclose(f);
      err = "w90g_read_mmn_device: pinned allocation failed";
      return 2;
    }
    const size_t got = std::fread(h_txt, 1, n, f);
    std::fclose(f);
    if (got != n) {
      cudaFreeHost(h_txt);
      err = std::string("Error: Problem reading input file ") + path;
      return 6;
    }
    if (h_txt[n - 1] != '\n') h_txt[n++] = '\n';
  }
  {
    // header record: counts as overlap_read checks them
    int hdr[3] = {0, 0, 0};
    const char* p = (const char*)std::memchr(h_txt, '\n', n);
    const char* q = p ? (const char*)std::memchr(p + 1, '\n', n - (size_t)(p + 1 - h_txt)) : nullptr;
    const std::string line = q ? std::string(p + 1, q) : std::string();
    if (!q || std::sscanf(line.c_str(), "%d %d %d", &hdr[0], &hdr[1], &hdr[2]) != 3) {
      err = std::string("Error: Problem reading input file ") + path;
      rc = 6;
      goto done;
    }
    if (hdr[0] != nb) err = std::string(path) + " has not the right number of bands";
    else if (hdr[1] != nk) err = std::string(path) + " has not the right number of k-points";
    else if (hdr[2] != nntot) err = std::string(path) + " has not the right number of nearest neighbours";
    if (!err.empty()) {
      rc = 6;
      goto done;
    }
  }
  {
    const int nc = (int)((n + kChunk - 1) / kChunk);
    SEED_CHECK(cudaMallocAsync((void**)&d_txt, n, st));
    SEED_CHECK(cudaMallocAsync((void**)&d_counts, (size_t)nc * 4, st));
    SEED_CHECK(cudaMallocAsync((void**)&d_flags, 4, st));
    SEED_CHECK(cudaMallocAsync((void**)&d_total, 4, st));
    SEED_CHECK(cudaMemsetAsync(d_flags, 0, 4, st));
    if (timing3) cudaEventRecord(ev[0], st);
    SEED_CHECK(cudaMemcpyAsync(d_txt, h_txt, n, cudaMemcpyHostToDevice, st));
    if (timing3) cudaEventRecord(ev[1], st);
    k_seed_count<<<nc, 256, 0, st>>>(d_txt, n, d_counts);
    k_seed_scan<<<1, 1024, 0, st>>>(d_counts, nc, d_total);
    *launches += 2;
    SEED_CHECK(cudaGetLastError());
    SEED_CHECK(cudaMemcpyAsync(&h_total, d_total, 4, cudaMemcpyDeviceToHost, st));
    SEED_CHECK(cudaStreamSynchronize(st));
    // records = newlines (the file ends with one); any extra records must be blank
    if ((long long)h_total < nrec_needed) {
      err = std::string("Error: Problem reading input file ") + path;
      rc = 6;
      goto done;
    }
    SEED_CHECK(cudaMallocAsync((void**)&d_starts, ((size_t)h_total + 1) * 8, st));
    k_seed_starts<<<nc, 32, 0, st>>>(d_txt, n, d_counts, d_starts);
    // blank records anywhere after the title line send the file to the host reader
    k_seed_blank<<<1024, 256, 0, st>>>(d_txt, d_starts, (long long)h_total, 1, d_flags);
    SEED_CHECK(cudaMallocAsync((void**)&d_dest, (size_t)nblk * 4, st));
    SEED_CHECK(cudaMallocAsync((void**)&d_nnl, (size_t)nblk * 4, st));
    SEED_CHECK(cudaMallocAsync((void**)&d_ncell, (size_t)nblk * 12, st));
    SEED_CHECK(cudaMemcpyAsync(d_nnl, nnlist, (size_t)nblk * 4, cudaMemcpyHostToDevice, st));
    SEED_CHECK(cudaMemcpyAsync(d_ncell, nncell, (size_t)nblk * 12, cudaMemcpyHostToDevice, st));
    k_mmn_heads<<<(unsigned)((nblk + 255) / 256), 256, 0, st>>>(d_txt, d_starts, nk, nntot, per, d_nnl, d_ncell,
                                                               d_dest, d_flags);
    *launches += 3;   // starts, blank, heads
    SEED_CHECK(cudaGetLastError());
    dest.resize((size_t)nblk);
    SEED_CHECK(cudaMemcpyAsync(dest.data(), d_dest, (size_t)nblk * 4, cudaMemcpyDeviceToHost, st));
    SEED_CHECK(cudaMemcpyAsync(&h_flags, d_flags, 4, cudaMemcpyDeviceToHost, st));
    SEED_CHECK(cudaStreamSynchronize(st));
    if (h_flags) {
      fallback = true;
    } else {
      std::vector<char> seen((size_t)nblk, 0);
      for (int d : dest) {
        if (seen[(size_t)d]) fallback = true;   // two blocks for one slot: host reader
        seen[(size_t)d] = 1;
      }
    }
    if (!fallback) {
      if (timing3) cudaEventRecord(ev[2], st);
      k_mmn_values<<<4 * 152 * 8, 256, 0, st>>>(d_txt, d_starts, nblk, per, (long long)nb * nb, d_dest,
                                               (double2*)d_m, d_flags);
      if (timing3) cudaEventRecord(ev[3], st);
      *launches += 1;
      SEED_CHECK(cudaGetLastError());
      SEED_CHECK(cudaMemcpyAsync(&h_flags, d_flags, 4, cudaMemcpyDeviceToHost, st));
      SEED_CHECK(cudaStreamSynchronize(st));
      fallback = h_flags != 0;
      if (timing3 && !fallback) {
        float a = 0.f, b = 0.f, c = 0.f;
        cudaEventElapsedTime(&a, ev[2], ev[3]);   // k_mmn_values
        cudaEventElapsedTime(&b, ev[1], ev[3]);   // all parse kernels and the host sync between them
        cudaEventElapsedTime(&c, ev[0], ev[1]);   // the text copy
        timing3[0] = a;
        timing3[1] = b;
        timing3[2] = c;
      }
    }
    *used_gpu = fallback ? 0 : 1;
  }
  if (fallback) {
    // host reader into pinned memory, then one copy to the device
    std::vector<double> m((size_t)2 * nblk * nb * nb, 0.0);
    rc = read_mmn(path, nb, nk, nntot, nnlist, nncell, m.data(), 0, err);
    if (rc == 0) SEED_CHECK(cudaMemcpyAsync(d_m, m.data(), m.size() * 8, cudaMemcpyHostToDevice, st));
    if (rc == 0) SEED_CHECK(cudaStreamSynchronize(st));
  }
done:
  if (d_txt) cudaFreeAsync(d_txt, st);
  if (d_counts) cudaFreeAsync(d_counts, st);
  if (d_flags) cudaFreeAsync(d_flags, st);
  if (d_total) cudaFreeAsync(d_total, st);
  if (d_starts) cudaFreeAsync(d_starts, st);
  if (d_dest) cudaFreeAsync(d_dest, st);
  if (d_nnl) cudaFreeAsync(d_nnl, st);
  if (d_ncell) cudaFreeAsync(d_ncell, st);
  cudaStreamSynchronize(st);
  if (h_txt) cudaFreeHost(h_txt);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  return rc;
}

}  // namespace w90g
