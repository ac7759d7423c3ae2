// Parallel readers of the formatted seed files (.mmn, .amn, .eig).
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace w90g {

// m: complex (nb, nb, nntot, nk) column-major, interleaved; nnlist [k][nn] 0-based,
// nncell [k][nn][3].  Returns 0, or 6 (file error) with err set.
int read_mmn(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell, double* m,
             int nthreads, std::string& err);
// a: complex (nb, nproj, nk)
int read_amn(const char* path, int nb, int nproj, int nk, double* a, int nthreads, std::string& err);
// eig: (nb, nk)
int read_eig(const char* path, int nb, int nk, double* eig, std::string& err);
// .mmn parsed on the GPU into device memory d_m (same layout as read_mmn); files outside
// the device parser's fast path go through read_mmn and one copy (*used_gpu = 0).
// *launches: kernels launched.  timing3 (nullable): ms of k_mmn_values, of all parse
// kernels, of the text copy (CUDA events on st).  Returns 0, 1 (CUDA), 2 (allocation) or
// 6 (file).
int read_mmn_device(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell, double* d_m,
                    cudaStream_t st, int* used_gpu, long long* launches, double* timing3, std::string& err);

}  // namespace w90g
