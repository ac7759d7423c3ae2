// Parallel readers of the formatted seed files (.mmn, .amn, .eig).
#pragma once
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

}  // namespace w90g
