// SIMT emulation of the disentanglement kernels (dis.cu), plain and symmetry-adapted, for
// the CPU tests: the kernel part of dis.cu (everything before dis_run; the test writes a
// copy in which `extern __shared__` arrays read emu_dyn_smem()) on the fiber launcher,
// replayed in dis_run's launch order with the C ABI's symmetry tables.
// the standard headers dis.cu includes come first: after the stand-in's qualifier macros
// they would no longer parse
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "emu_fibers.h"

#include "dis_emu.cu"
#include "sym_tables.h"

extern "C" {

// eig (nb, K), Mraw (nb, nb, B, K), A (nb, W, K): Fortran order, complex interleaved.
// Outputs: log rows (iter, Omega_I(i-1), Omega_I(i)), U0 (W, W, K), M0 (W, W, B, K),
// U_opt (nb, W, K); status[0] = 0 or the first failure.  threads: CUDA threads per CTA
// (the engine launches 256; the kernels take any power of two).  Returns the iterations run.
int emu_dis_sym(int nb, int W, int K, int B, const int* nnlist, const double* wb, double wbtot, const double* eig,
                const double* Mraw, const double* A, int num_iter, double mix, double conv_tol, int conv_window,
                double win_min, double win_max, int nsym, int nkirr, const int* ik2ir, const int* ir2ik,
                const int* kptsym, const double* dw, const double* db, double eps, int threads, double* log_out,
                double* U0_out, double* M0_out, double* Uopt_out, int* status_out) {
  using namespace w90g;
  DisControl c;
  c.num_iter = num_iter;
  c.mix_ratio = mix;
  c.conv_tol = conv_tol;
  c.conv_window = conv_window;
  c.win_min = win_min;
  c.win_max = win_max;
  std::vector<int> ndim, nfirst, nfroz, ffirst, nfidx;
  std::vector<double> eigw;
  std::string err;
  if (int rc = dis_windows(c, eig, nb, W, K, ndim, nfirst, nfroz, ffirst, nfidx, eigw, err)) return -100 - rc;
  SymTables t;
  if (int rc = build_sym_tables(W, nb, nsym, nkirr, K, ik2ir, ir2ik, kptsym, dw, db, t, err)) return -200 - rc;
  const size_t NN = (size_t)nb * nb, WW = (size_t)W * W;
  std::vector<int> nn(nnlist, nnlist + (size_t)K * B), st(K, 0), sw(1, 0), ints;
  std::vector<double> wbv(wb, wb + B), wk1(K), wk(K);
  std::vector<double2> mraw((size_t)K * B * NN), mw((size_t)K * B * NN), a((size_t)K * nb * W), u0b((size_t)K * nb * W),
      u1b((size_t)K * nb * W), zin((size_t)K * NN), zout((size_t)K * NN), uw((size_t)K * WW), m0((size_t)K * B * WW),
      ws((size_t)K * kWs * NN), vz((size_t)K * NN), syws((size_t)t.nir * kDisSymWs * NN);
  std::memcpy(mraw.data(), Mraw, mraw.size() * 16);
  std::memcpy(u0b.data(), A, u0b.size() * 16);
  for (auto* v : {&t.ik, &t.moff, &t.mem, &t.goff, &t.grp}) ints.insert(ints.end(), v->begin(), v->end());
  ints.insert(ints.end(), (size_t)t.nir, 0);
  DisDev D{};
  D.nb = nb;
  D.W = W;
  D.K = K;
  D.B = B;
  D.wbtot = wbtot;
  D.mix = mix;
  D.nnlist = nn.data();
  D.wb = wbv.data();
  D.ndim = ndim.data();
  D.nfirst = nfirst.data();
  D.nfroz = nfroz.data();
  D.ffirst = ffirst.data();
  D.nfidx = nfidx.data();
  D.eig = eigw.data();
  D.Mraw = mraw.data();
  D.Mw = mw.data();
  D.A = a.data();
  D.U[0] = u0b.data();
  D.U[1] = u1b.data();
  D.Zin = zin.data();
  D.Zout = zout.data();
  D.U0 = uw.data();
  D.M0 = m0.data();
  D.ws = ws.data();
  D.wk1 = wk1.data();
  D.wk = wk.data();
  D.status = st.data();
  D.Vz = vz.data();
  D.max_sweeps = sw.data();
  D.sym_nir = t.nir;
  D.sym_nsym = t.nsym;
  D.sym_eps = eps;
  size_t o = 0;
  D.sym_ik = ints.data();
  D.sym_moff = ints.data() + (o += t.ik.size());
  D.sym_mem = ints.data() + (o += t.moff.size());
  D.sym_goff = ints.data() + (o += t.mem.size());
  D.sym_grp = ints.data() + (o += t.goff.size());
  D.sym_status = ints.data() + (o += t.grp.size());
  D.sym_d = reinterpret_cast<const double2*>(t.d.data());
  D.sym_db = reinterpret_cast<const double2*>(t.db.data());
  D.sym_ws = syws.data();
  const int nir = t.nir;
  // dis_run's order, symmetry-adapted
  launch(K, threads, 0, [&] { k_dis_project(D); });
  int cur = 0, it = 0;
  launch(nir, threads, 0, [&] { k_dis_sym_u(D, cur, 0); });
  launch(K, threads, 0, [&] { k_dis_z(D, cur, 1, 0); });
  launch(nir, threads, 0, [&] { k_dis_sym_z(D, 0); });
  std::vector<double> history(conv_window, 0.0);
  int rows = 0;
  for (it = 1; it <= num_iter; ++it) {
    launch(nir, threads, 0, [&] { k_dis_sym_step(D, cur, it); });
    launch(nir, threads, 0, [&] { k_dis_sym_u(D, cur ^ 1, 0); });
    launch(K, threads, 0, [&] { k_dis_z(D, cur ^ 1, 0, 1); });
    launch(nir, threads, 0, [&] { k_dis_sym_z(D, 1); });
    cur ^= 1;
    double w1 = 0.0, w2 = 0.0;
    for (int k = 0; k < K; ++k) {
      w1 += wk1[k];
      w2 += wk[k];
    }
    w1 /= K;
    w2 /= K;
    log_out[3 * rows] = it;
    log_out[3 * rows + 1] = w1;
    log_out[3 * rows + 2] = w2;
    ++rows;
    const double delta = w1 / w2 - 1.0;
    if (conv_window == 0) {
    } else if (it <= conv_window) {
      history[it - 1] = delta;
    } else {
      for (int i = 0; i + 1 < conv_window; ++i) history[i] = history[i + 1];
      history[conv_window - 1] = delta;
    }
    if (it >= conv_window) {
      bool conv = true;
      for (double h : history) conv = conv && std::fabs(h) < conv_tol;
      if (conv) break;
    }
  }
  launch(K, threads, 0, [&] { k_dis_findu(D, cur); });
  launch(nir, threads, 0, [&] { k_dis_sym_u(D, cur, 1); });
  launch(K * B, threads, ((size_t)W * nb + 2 * WW) * 16, [&] { k_dis_rotate(D, cur); });
  status_out[0] = 0;
  for (int k = 0; k < K && !status_out[0]; ++k) status_out[0] = st[k];
  for (int i = 0; i < nir && !status_out[0]; ++i) status_out[0] = D.sym_status[i];
  std::memcpy(U0_out, uw.data(), uw.size() * 16);
  std::memcpy(M0_out, m0.data(), m0.size() * 16);
  std::memcpy(Uopt_out, D.U[cur], u0b.size() * 16);
  return rows;
}

// The same without symmetry (dis_run's plain order, frozen states included): k_dis_project,
// k_dis_froz, k_dis_z, the k_dis_step / k_dis_z iterations, k_dis_gauge, k_dis_findu,
// k_dis_rotate.  Same arguments as emu_dis_sym minus the symmetry data, plus the frozen
// window.
int emu_dis_plain(int nb, int W, int K, int B, const int* nnlist, const double* wb, double wbtot, const double* eig,
                  const double* Mraw, const double* A, int num_iter, double mix, double conv_tol, int conv_window,
                  double win_min, double win_max, int frozen, double froz_min, double froz_max, int threads,
                  double* log_out, double* U0_out, double* M0_out, double* Uopt_out, int* status_out) {
  using namespace w90g;
  DisControl c;
  c.num_iter = num_iter;
  c.mix_ratio = mix;
  c.conv_tol = conv_tol;
  c.conv_window = conv_window;
  c.win_min = win_min;
  c.win_max = win_max;
  c.frozen_states = frozen != 0;
  c.froz_min = froz_min;
  c.froz_max = froz_max;
  std::vector<int> ndim, nfirst, nfroz, ffirst, nfidx;
  std::vector<double> eigw;
  std::string err;
  if (int rc = dis_windows(c, eig, nb, W, K, ndim, nfirst, nfroz, ffirst, nfidx, eigw, err)) return -100 - rc;
  const size_t NN = (size_t)nb * nb, WW = (size_t)W * W;
  std::vector<int> nn(nnlist, nnlist + (size_t)K * B), st(K, 0), sw(1, 0);
  std::vector<double> wbv(wb, wb + B), wk1(K), wk(K);
  std::vector<double2> mraw((size_t)K * B * NN), mw((size_t)K * B * NN), a((size_t)K * nb * W), u0b((size_t)K * nb * W),
      u1b((size_t)K * nb * W), zin((size_t)K * NN), zout((size_t)K * NN), uw((size_t)K * WW), m0((size_t)K * B * WW),
      ws((size_t)K * kWs * NN), vz((size_t)K * NN);
  std::memcpy(mraw.data(), Mraw, mraw.size() * 16);
  std::memcpy(u0b.data(), A, u0b.size() * 16);
  DisDev D{};
  D.nb = nb;
  D.W = W;
  D.K = K;
  D.B = B;
  D.wbtot = wbtot;
  D.mix = mix;
  D.nnlist = nn.data();
  D.wb = wbv.data();
  D.ndim = ndim.data();
  D.nfirst = nfirst.data();
  D.nfroz = nfroz.data();
  D.ffirst = ffirst.data();
  D.nfidx = nfidx.data();
  D.eig = eigw.data();
  D.Mraw = mraw.data();
  D.Mw = mw.data();
  D.A = a.data();
  D.U[0] = u0b.data();
  D.U[1] = u1b.data();
  D.Zin = zin.data();
  D.Zout = zout.data();
  D.U0 = uw.data();
  D.M0 = m0.data();
  D.ws = ws.data();
  D.wk1 = wk1.data();
  D.wk = wk.data();
  D.status = st.data();
  D.Vz = vz.data();
  D.max_sweeps = sw.data();
  bool any_froz = false;
  int mmax = 0;
  for (int k = 0; k < K; ++k) {
    any_froz = any_froz || nfroz[k] > 0;
    mmax = std::max(mmax, ndim[k] - nfroz[k]);
  }
  const size_t step_smem = 3 * (size_t)mmax * mmax * 16;
  launch(K, threads, 0, [&] { k_dis_project(D); });
  if (any_froz) launch(K, threads, 0, [&] { k_dis_froz(D); });
  int cur = 0, it = 0, rows = 0;
  launch(K, threads, 0, [&] { k_dis_z(D, cur, 1, 0); });
  std::vector<double> history(conv_window, 0.0);
  for (it = 1; it <= num_iter; ++it) {
    launch(K, threads, step_smem, [&] { k_dis_step(D, cur, it); });
    launch(K, threads, 0, [&] { k_dis_z(D, cur ^ 1, 0, 1); });
    cur ^= 1;
    double w1 = 0.0, w2 = 0.0;
    for (int k = 0; k < K; ++k) {
      w1 += wk1[k];
      w2 += wk[k];
    }
    w1 /= K;
    w2 /= K;
    log_out[3 * rows] = it;
    log_out[3 * rows + 1] = w1;
    log_out[3 * rows + 2] = w2;
    ++rows;
    const double delta = w1 / w2 - 1.0;
    if (conv_window == 0) {
    } else if (it <= conv_window) {
      history[it - 1] = delta;
    } else {
      for (int i = 0; i + 1 < conv_window; ++i) history[i] = history[i + 1];
      history[conv_window - 1] = delta;
    }
    if (it >= conv_window) {
      bool conv = true;
      for (double h : history) conv = conv && std::fabs(h) < conv_tol;
      if (conv) break;
    }
  }
  launch(K, threads, 0, [&] { k_dis_gauge(D, cur); });
  launch(K, threads, 0, [&] { k_dis_findu(D, cur); });
  launch(K * B, threads, ((size_t)W * nb + 2 * WW) * 16, [&] { k_dis_rotate(D, cur); });
  status_out[0] = 0;
  for (int k = 0; k < K && !status_out[0]; ++k) status_out[0] = st[k];
  std::memcpy(U0_out, uw.data(), uw.size() * 16);
  std::memcpy(M0_out, m0.data(), m0.size() * 16);
  std::memcpy(Uopt_out, D.U[cur], u0b.size() * 16);
  return rows;
}

}  // extern "C"
