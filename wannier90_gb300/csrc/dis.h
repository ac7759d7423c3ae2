// Host side of the GPU disentanglement (dis_main + setup_m_loc of the reference).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace w90g {

constexpr int kDisLogStride = 5;

struct DisControl {
  int num_iter = 200;            // dis_num_iter
  double mix_ratio = 0.5;        // dis_mix_ratio
  double conv_tol = 1.0e-10;     // dis_conv_tol
  int conv_window = 3;           // dis_conv_window
  double win_min = -1.0e300, win_max = 1.0e300;     // outer window (eV)
  double froz_min = -1.0e300, froz_max = 1.0e300;   // inner (frozen) window (eV)
  bool frozen_states = false;    // dis_froz_max given
};

// kernels of the disentanglement, in the order of DisSpec::prof_ms
enum DisKernel { kDisProject = 0, kDisFroz, kDisZ, kDisStep, kDisGauge, kDisFindU, kDisRotate, kDisSym, kDisKernels };
const char* dis_kernel_name(int i);

struct DisSpec {
  int nb = 0, W = 0, K = 0, B = 0;
  double wbtot = 0.0;
  std::vector<int> nnlist;       // [k][b] 0-based
  std::vector<double> wb;        // [b]
  // inputs, host or device memory (kind); eig is read on the host for the windows
  const double* eig = nullptr;   // eigval(nb, K)
  const double* M = nullptr;     // m_matrix(nb, nb, B, K), complex interleaved
  const double* A = nullptr;     // projections u_opt(nb, W, K), complex interleaved
  // outputs, same memory kind: U_opt (nb, W, K), U (W, W, K), and the top-left W x W of
  // each nb x nb block of m_out (may alias M)
  double* uopt_out = nullptr;
  double* u_out = nullptr;
  double* m_out = nullptr;
  bool device = false;           // pointers are device memory
  cudaStream_t stream = nullptr; // 0: a private stream
  DisControl ctl;
  // per-kernel device time (ms, CUDA events around each launch) and launch counts,
  // indexed by DisKernel; null = no timing
  double* prof_ms = nullptr;
  int* prof_counts = nullptr;
  // symmetry-adapted mode (site_symmetry = T): the tables of w90g_set_sitesym with the
  // band slots nb x nb (sym_db) and the Wannier slots W x W (sym_d); sym_nir = 0: off
  int sym_nir = 0, sym_nsym = 0;
  double sym_eps = 1.0e-3;
  std::vector<int> sym_ik, sym_moff, sym_mem, sym_goff, sym_grp;
  std::vector<double> sym_d, sym_db;
};

struct DisResult {
  std::vector<int> ndimwin, nfirstwin;
  double omega_invariant = 0.0;
  std::vector<double> log;       // rows of kDisLogStride: (iter, Omega_I(i-1), Omega_I(i), delta, seconds)
  int converged = 0;
  long long launches = 0;
  int max_sweeps = 0;            // Jacobi sweeps of the Z eigenproblems, max over k and iterations
};

// Returns 0, or an ierr code (1 fatal / 2 allocation / 5 input) with err set.
int dis_run(const DisSpec& s, DisResult& r, std::string& err);

}  // namespace w90g
