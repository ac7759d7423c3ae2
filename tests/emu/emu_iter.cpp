// SIMT emulation of the FP64 wann_main iteration (k_fp64.cu) with the symmetry-adapted
// kernels (k_sitesym.cu), for the CPU tests.  The threads of a CTA are fibers (ucontext)
// of one host thread: each runs until its next __syncthreads, and the barrier opens once
// every fiber has arrived or returned; CTAs run one after another.  The test compiles
// copies of the kernel sources in which `extern __shared__` arrays read emu_dyn_smem()
// and the %globaltimer read is 0 (the only two edits); everything else is the kernel
// source as the GPU builds it.  emu_wann_main replays the engine's launch order
// (Engine::project, Engine::begin, Engine::launch_iteration) for one problem on the FP64
// path (W <= 32).
#include "emu_fibers.h"

#include "k_fp64_emu.cu"
#include "k_sitesym.cu"
#include "sym_tables.h"

extern "C" {

// M (K*B blocks W x W) and A (K blocks) column-major complex; tables as for
// w90g_set_sitesym (nsym = 0: no symmetry); slwf_num > 0: selective localisation with
// lambda and the constrained centres [3][W] (null: unconstrained).  Writes log ((num_iter+1) x kLogStride),
// the final U (K blocks), status[2] = (projection status, unitarity/other).
// Returns the number of log rows.
int emu_wann_main(int W, int K, int B, const int* nnlist, const double* bk, const double* wb, double wbtot,
                  const double* Mraw, const double* A, int num_iter, int num_cg_steps, int conv_window,
                  double conv_tol, double trial_step, int nsym, int nkirr, const int* ik2ir, const int* ir2ik,
                  const int* kptsym, const double* dw, const double* db, double eps, int slwf_num, double slwf_lambda,
                  const double* slwf_c, double* log_out, double* U_out, int* status) {
  using namespace w90g;
  const size_t WW = (size_t)W * W, KB = (size_t)K * B;
  const int nt = (W + 31) / 32, ntt = nt * nt;
  const int nchunk = (int)((KB + 63) / 64);
  std::vector<double2> M0(KB * WW), M1(KB * WW), U0(K * WW), U1(K * WW), G(K * WW), D(K * WW), dU(K * WW);
  std::memcpy(M0.data(), Mraw, KB * WW * 16);
  std::memcpy(U0.data(), A, K * WW * 16);
  std::vector<double> dln(KB * W), dab(KB * W), offd(KB), gpart((size_t)K * ntt * 2), cen(12 * W),
      logv((size_t)(num_iter + 1) * kLogStride), logc((size_t)(num_iter + 1) * 4 * W), op1((size_t)nchunk * (4 * W + 2)),
      op2(nchunk), bkv(bk, bk + KB * 3), wbv(wb, wb + B);
  std::vector<int> nn(nnlist, nnlist + KB), st_lowdin(K, 0);
  CtrlState st{};
  st.cur = 0;
  st.first_pass = 1;
  st.lfirst = 1;
  Problem P{};
  P.W = W;
  P.K = K;
  P.B = B;
  P.wbtot = wbtot;
  P.M[0] = M0.data();
  P.M[1] = M1.data();
  P.U[0] = U0.data();
  P.U[1] = U1.data();
  P.G = G.data();
  P.D = D.data();
  P.dU = dU.data();
  P.nnlist = nn.data();
  P.bk = bkv.data();
  P.wb = wbv.data();
  P.diag_ln = dln.data();
  P.diag_abs2 = dab.data();
  P.offd = offd.data();
  P.gpart = gpart.data();
  P.centres = cen.data();
  P.log = logv.data();
  P.log_centres = logc.data();
  P.opart1 = op1.data();
  P.opart2 = op2.data();
  P.nchunk = nchunk;
  P.st = &st;
  P.ctl.num_iter = num_iter;
  P.ctl.num_cg_steps = num_cg_steps;
  P.ctl.conv_window = conv_window;
  P.ctl.conv_tol = conv_tol;
  P.ctl.trial_step = trial_step;
  P.ctl.conv_noise_amp = -1.0;
  // symmetry tables in the engine's layout (Engine::set_sym)
  SymTables t;
  std::vector<int> ints;
  std::vector<double> work;
  if (nsym > 0) {
    std::string msg;
    if (int rc = build_sym_tables(W, W, nsym, nkirr, K, ik2ir, ir2ik, kptsym, dw, db, t, msg)) return -rc;
    for (auto* v : {&t.ik, &t.moff, &t.mem, &t.goff, &t.grp}) ints.insert(ints.end(), v->begin(), v->end());
    ints.insert(ints.end(), (size_t)t.nir, 0);
    int* base = ints.data();
    size_t o = 0;
    P.sym_nir = t.nir;
    P.sym_eps = eps;
    P.sym_ik = base;
    P.sym_moff = base + (o += t.ik.size());
    P.sym_mem = base + (o += t.moff.size());
    P.sym_goff = base + (o += t.mem.size());
    P.sym_grp = base + (o += t.goff.size());
    P.sym_status = base + (o += t.grp.size());
    P.sym_d = reinterpret_cast<const double2*>(t.d.data());
    P.sym_db = reinterpret_cast<const double2*>(t.db.data());
    work.assign((size_t)t.nir * kSymWork * WW * 2, 0.0);
    P.sym_work = reinterpret_cast<double2*>(work.data());
  }
  // selective localisation (Engine::set_slwf): centres [3][W], lambda_loc, nu0
  std::vector<double> slwfc;
  if (slwf_num > 0) {
    P.slwf_num = slwf_num;
    slwfc.assign(3 * (size_t)W, 0.0);
    if (slwf_c) {
      slwfc.assign(slwf_c, slwf_c + 3 * (size_t)W);
      P.slwf_lambda = slwf_lambda;
      double c2 = 0.0;
      for (int n = 0; n < slwf_num; ++n)
        for (int i = 0; i < 3; ++i) c2 += slwfc[(size_t)i * W + n] * slwfc[(size_t)i * W + n];
      P.slwf_nu0 = slwf_lambda * c2;
    }
    P.slwf_c = slwfc.data();
  }
  int offs_k[2] = {0, K}, offs_kb[2] = {0, (int)KB}, offs_grad[2] = {0, K * ntt}, offs_chunk[2] = {0, nchunk},
      offs_ir[2] = {0, P.sym_nir};
  const WorkMap wmk{offs_k, 1}, wmkb{offs_kb, 1}, wmg{offs_grad, 1}, wmc{offs_chunk, 1}, wmir{offs_ir, 1};
  const size_t sm4 = 4 * WW * 16, sm6 = 6 * WW * 16;
  Problem* pp = &P;
  auto omega = [&](int slot) {
    launch(nchunk, 256, 0, [&] { k_omega_p1(pp, wmc, slot); });
    launch(nchunk, 256, 0, [&] { k_omega_p2(pp, wmc, slot); });
  };
  // Engine::project
  launch(K, 256, sm4, [&] { k_lowdin(pp, wmk, st_lowdin.data()); });
  if (P.sym_nir) launch(P.sym_nir, 256, 0, [&] { k_sym_u(pp, wmir); });
  status[0] = 0;
  for (int k = 0; k < K; ++k) status[0] |= st_lowdin[k];
  for (int i = 0; i < P.sym_nir; ++i) status[0] |= P.sym_status[i] << 4;
  launch((int)KB, 256, sm4, [&] { k_m_update(pp, wmkb, 1, 0); });
  // Engine::begin
  launch((int)KB, 128, 0, [&] { k_mdiag(pp, wmkb); });
  omega(2);
  launch(1, 128, 0, [&] { k_log_init(pp); });
  // Engine::launch_iteration, until the controller stops
  for (int it = 0; it < num_iter && !st.done; ++it) {
    launch(K * ntt, 256, 0, [&] { k_grad(pp, wmg); });
    if (P.sym_nir) launch(P.sym_nir, 256, 0, [&] { k_sym_grad(pp, wmir); });
    launch(1, 256, 0, [&] { k_ctrl_search(pp); });
    if (P.sym_nir) launch(P.sym_nir, 256, 0, [&] { k_sym_dir(pp, wmir); });
    launch(K, 256, sm6, [&] { k_exp_u(pp, wmk, 0); });
    launch((int)KB, 256, sm4, [&] { k_m_update(pp, wmkb, 0, 0); });
    omega(0);
    launch(1, 128, 0, [&] { k_ctrl_step(pp, 1); });
    launch(K, 256, sm6, [&] { k_exp_u(pp, wmk, 1); });
    launch((int)KB, 256, sm4, [&] { k_m_update(pp, wmkb, 0, 1); });
    omega(1);
    launch(1, 128, 0, [&] { k_ctrl_end(pp); });
  }
  status[1] = st.error;
  const int rows = st.iter + 1;
  std::memcpy(log_out, logv.data(), (size_t)rows * kLogStride * 8);
  std::memcpy(U_out, P.U[st.cur], K * WW * 16);
  return rows;
}

}  // extern "C"
