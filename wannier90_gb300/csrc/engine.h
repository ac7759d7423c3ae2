// Host orchestration of the GB300 MLWF engine: device arena, launch sequence,
// CUDA-graph replay of the iteration, result download.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "w90g.cuh"

namespace w90g {

struct ProblemSpec {
  int W = 0, K = 0, B = 0;
  double wbtot = 0.0;
  std::vector<int> nnlist;   // [k][b] 0-based
  std::vector<double> bk;    // [k][b][3]
  std::vector<double> wb;    // [b]
  Control ctl{};
  int tensor = 0;            // request the tensor-core M update (W <= 128)
  int tensor_exp = 1;        // with tensor: exp(s D) and U dU on the tensor cores too
  int mupdate_pipe = 1;      // with tensor and W <= 32: the pipelined M-update kernel (k_mupdate2.cu)
  int exp_smem = 0;          // with tensor exp and 16 < W <= 32: the exp chain's matrices in shared memory
  // preconditioner (precond = T): Wigner-Seitz points R_r of the Born-von Karman
  // supercell, exp(-i 2 pi k.R) table [k][r] (re, im interleaved), |R|^2, degeneracies
  int precond = 0;
  int nrpts = 0;
  std::vector<double> pc_kr, pc_r2, pc_ndeg;
  // guiding centres: initial centres [3][W] (Cartesian, Angstrom), b directions and
  // their neighbour indices (kmesh_info nnh, bka, neigh)
  int guiding = 0, no_guide_iter = 0, guide_cycles = 1, nnh = 0;
  std::vector<double> rguide0, bka;
  std::vector<int> neigh;
  // selective localisation: slwf_num objective WFs (0 = off, i.e. slwf_num = num_wann),
  // lambda_loc, constrained centres [3][W] (Cartesian, Angstrom; empty = unconstrained)
  int slwf_num = 0;
  double slwf_lambda = 0.0;
  std::vector<double> slwf_c;
  // symmetry-adapted mode (isolated bands): the tables of Problem::sym_* (sym_nir = 0:
  // off); sym_d / sym_db hold the slot matrices, W x W column-major, re/im interleaved
  int sym_nir = 0;
  double sym_eps = 1.0e-3;
  std::vector<int> sym_ik, sym_moff, sym_mem, sym_goff, sym_grp;
  std::vector<double> sym_d, sym_db;
};

struct ProblemResult {
  int niter = 0;
  int converged = 0;
  int error = 0;
  Spread spread{};
  std::vector<double> centres;   // [W][3]
  std::vector<double> spreads;   // [W]
  std::vector<double> log;       // (niter+1) x kLogStride
  std::vector<double> log_centres;  // (niter+1) x 4W
  double unitarity_err = 0.0;
};

enum ProfKernel {
  kPGrad = 0, kPCtrlSearch, kPExpU, kPMUpdate, kPOmega, kPCtrlStep, kPCtrlEnd, kPInit, kPPrecond, kPNum
};
extern const char* kProfNames[kPNum];

class Engine {
 public:
  Engine();
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  // (Re)allocate for a batch of problems; reuses the arena when the shapes match.
  int setup(const std::vector<ProblemSpec>& specs, std::string& err);
  // Copy M (m_matrix layout) and U into buffer 0 of problem p.  ldm > W reads the
  // top-left W x W of ldm x ldm blocks (m_matrix_local after disentanglement).
  int load(int p, const void* M, const void* U, cudaMemcpyKind kind, std::string& err, int ldm = 0);
  // Copy the accepted M and U of problem p out (into the top-left W x W for ldm > W).
  int store(int p, void* M, void* U, cudaMemcpyKind kind, std::string& err, int ldm = 0);
  // Loewdin projection on every problem (U holds A on entry).
  int project(std::string& err);
  // wann_main on every problem; results via result().  Equivalent to begin(), advance()
  // until every problem is done, finish().
  int wannierise(std::string& err);
  // Stepwise form (used by the serving loop): begin() computes the initial spread and
  // captures the iteration graph; advance(n, d_flag) enqueues n more iterations and, if
  // d_flag is given, a kernel that sets *d_flag = 1 once every problem is done;
  // finish() runs the final rotation/unitarity check and downloads the results.
  // All work is enqueued on stream(); nothing here synchronises except finish().
  int begin(std::string& err);
  int advance(int n, int* d_flag, std::string& err);
  int finish(std::string& err);
  int launched_iters() const { return launched_iters_; }
  int max_iter() const { return max_iter_; }
  size_t arena_bytes() const { return arena_bytes_; }
  // device bytes setup() would allocate for these problems (HBM admission)
  static size_t estimate_bytes(const std::vector<ProblemSpec>& specs);
  // wann_main with each kernel launched individually and timed with CUDA events on the
  // launching stream; ms[i] / cnt[i] accumulate per kernel kind (kProfNames order);
  // only launches that did work are counted (skipped second passes are excluded).
  int wannierise_profiled(int max_iters, double* ms, int* cnt, std::string& err);
  const ProblemResult& result(int p) const { return results_[p]; }
  int nprob() const { return (int)specs_.size(); }

  void set_stream(cudaStream_t s) { user_stream_ = s; }
  // allocate / free the arena stream-ordered on stream() (the stream must outlive the
  // engine); avoids the device-wide synchronisation of cudaFree in the serving loop
  void set_async_alloc(bool on) { async_alloc_ = on; }
  cudaStream_t stream() const { return user_stream_ ? user_stream_ : own_stream_; }
  long long launches() const { return launches_; }
  double last_exp_products() const { return last_exp_products_; }

 private:
  int alloc(std::string& err);
  void release();
  void launch_iteration(cudaStream_t s);
  void launch_omega(cudaStream_t s, int slot);
  void launch_mupdate(cudaStream_t s, int which);
  void launch_exp(cudaStream_t s, int which);
  int prepare_tensor(cudaStream_t st, std::string& err);
  int init_states(std::string& err);
  int set_slwf(int p, std::string& err);
  int set_sym(int p, std::string& err);

  std::vector<ProblemSpec> specs_;
  std::vector<Problem> hprobs_;
  std::vector<ProblemResult> results_;
  void* arena_ = nullptr;
  size_t arena_bytes_ = 0;
  Problem* dprobs_ = nullptr;
  int* d_offs_k_ = nullptr;
  int* d_offs_kb_ = nullptr;
  int* d_offs_grad_ = nullptr;
  int* d_offs_chunk_ = nullptr;
  int* d_status_ = nullptr;
  double* d_unit_ = nullptr;
  int n_k_ = 0, n_kb_ = 0, n_grad_ = 0, n_chunk_ = 0;
  int n_ir_ = 0;         // irreducible k-points of the symmetry-adapted problems (CTAs of k_sym_*)
  int* d_offs_ir_ = nullptr;
  int pc_tiles_ = 0;     // > 0: some problem is preconditioned; CTAs per problem of k_precond
  int guide_w_ = 0;      // > 0: some problem uses guiding centres; CTAs per problem of k_phases
  int maxW_small_ = 0;   // largest W <= 32 in the batch (shared-memory kernels)
  int tensor_wp_ = 0;    // > 0: tensor M update with padded width 8..128 for the whole batch
  bool tensor_exp_ = false;  // exp(s D) on the tensor cores (k_oz_exp)
  bool pipe_ = false;        // tensor M update by the pipelined kernel (tensor_wp_ <= 32)
  bool exp_smem_ = false;    // tensor exp with its FP64 matrices in shared memory (tensor_wp_ == 32)
  int max_iter_ = 0;
  cudaStream_t own_stream_ = nullptr;
  cudaStream_t user_stream_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  cudaStream_t graph_stream_ = nullptr;
  std::string layout_key_;
  long long launches_ = 0;
  int launched_iters_ = 0;
  std::vector<double> guide_init_;   // host staging of csheet = 1
  std::vector<std::vector<double>> slwf_host_;   // host staging of the constrained centres
  std::vector<std::vector<int>> sym_host_;       // host staging of the symmetry tables
  bool async_alloc_ = false;
  double last_exp_products_ = 0.0;
};

int measure_fp64_peak(double* tflops, std::string& err);
size_t oz_smem_bytes(int wp);

}  // namespace w90g
