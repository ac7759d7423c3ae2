// Host side of the GPU disentanglement (dis_main + setup_m_loc of the reference).
#pragma once
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

struct DisSpec {
  int nb = 0, W = 0, K = 0, B = 0;
  double wbtot = 0.0;
  std::vector<int> nnlist;       // [k][b] 0-based
  std::vector<double> wb;        // [b]
  const double* eig = nullptr;   // eigval(nb, K)
  const double* M = nullptr;     // m_matrix(nb, nb, B, K), complex interleaved
  const double* A = nullptr;     // projections u_opt(nb, W, K), complex interleaved
  DisControl ctl;
};

struct DisResult {
  std::vector<double> u_opt;     // (nb, W, K) complex: optimal subspace in window rows
  std::vector<double> u;         // (W, W, K) complex: internal_find_u
  std::vector<double> m;         // (W, W, B, K) complex: U^H U_opt^H M U_opt' U'
  std::vector<int> ndimwin, nfirstwin;
  double omega_invariant = 0.0;
  std::vector<double> log;       // rows of kDisLogStride: (iter, Omega_I(i-1), Omega_I(i), delta, seconds)
  int converged = 0;
};

// Returns 0, or an ierr code (1 fatal / 2 allocation / 5 input) with err set.
int dis_run(const DisSpec& s, DisResult& r, std::string& err);

}  // namespace w90g
