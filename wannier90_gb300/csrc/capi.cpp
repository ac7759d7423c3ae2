// C ABI of the GB300 MLWF engine (declared in include/wannier90_gb300.h).
//
// Mirrors Wannier90's library flow (src/library_interface.F90, src/c_interface.F90):
//   w90_create -> cset_option_* -> cinput_setopt (parse options, build the k-mesh)
//   -> cget_nn / cget_nnkp -> cset_m_local / cset_u_matrix / cset_u_opt
//   -> cproject_overlap -> cwannierise -> cget_centres / cget_spreads -> w90_delete
// All compute of cproject_overlap / cwannierise runs in the CUDA engine (engine.cu);
// there is no host compute path.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/wannier90_gb300.h"
#include "dis.h"
#include "engine.h"
#include "kmesh.h"
#include "seedio.h"
#include "sym_tables.h"
#include "winfile.h"

namespace {

using w90g::Control;
using w90g::Engine;
using w90g::KmeshInfo;
using w90g::ProblemSpec;

struct Opt {
  std::vector<double> v;
  int rows = 1, cols = 1;
  bool is_int = false;
};

struct Handle {
  std::map<std::string, Opt> opts;
  bool setup_complete = false;
  // system
  int num_wann = 0, num_bands = 0, num_kpts = 0;
  int mp_grid[3] = {0, 0, 0};
  double real_lattice[9] = {0};
  std::vector<double> kpt_latt;
  // knobs
  Control ctl{};
  int iprint = 1, num_print_cycles = 1, timing_level = 1;
  int search_shells = 36;
  double kmesh_tol = 1.0e-6;
  int gpu_tensor = 0;   // M update on tensor cores (W <= 128)
  int gpu_tensor_exp = 1;
  int gpu_mupdate_pipe = 1;   // tensor path, W <= 32: pipelined M-update kernel
  int gpu_exp_smem = 0;       // tensor exp, 16 < W <= 32: matrices in shared memory
  KmeshInfo km;
  // preconditioner tables (precond = T), built at cinput_setopt like wann_main's
  // hamiltonian_setup / k_to_r (src/wannierise.F90:269-300)
  int precond = 0, nrpts = 0;
  std::vector<double> pc_kr, pc_r2, pc_ndeg;
  // guiding centres (wann_main :415-420, wann_phases); the centres are the projection
  // sites, passed as the engine option guiding_centres_frac (num_wann x 3, fractional)
  int guiding = 0, no_guide_iter = 0, guide_cycles = 1;
  std::vector<double> rguide0;   // [3][W] Cartesian
  // selective localisation (wann_slwf_type): slwf_num objective WFs (0 = off), lambda_loc
  // and the constrained centres [3][W] (Cartesian; empty = unconstrained), from slwf_num /
  // slwf_constrain / slwf_lambda and the engine option slwf_centres_frac (num_wann x 3,
  // fractional; the <slwf_centres> block merged over the projection sites)
  int slwf_num = 0;
  double slwf_lambda = 0.0;
  std::vector<double> slwf_c;
  // symmetry-adapted mode (site_symmetry = T): the .dmn data as sitesym_read holds it,
  // set by w90g_set_sitesym, turned into the engine's tables (ProblemSpec::sym_*)
  int site_symmetry = 0;
  double symmetrize_eps = 1.0e-3;
  bool have_sym = false;
  int sym_nir = 0, sym_nk = 0, sym_nb = 0, sym_nsym = 0;
  std::vector<int> sym_ik, sym_moff, sym_mem, sym_goff, sym_grp;
  std::vector<double> sym_d, sym_db;
  // caller data
  double* m_local = nullptr;
  double* u_matrix = nullptr;
  double* u_opt = nullptr;
  double* eigval = nullptr;
  // disentanglement (dis_main + setup_m_loc, src/library_interface.F90:362-420)
  w90g::DisControl dis_ctl;
  bool have_disentangled = false;
  double omega_invariant = 0.0;
  int dis_converged = 0;
  std::vector<double> dis_log;
  long long dis_launches = 0;
  int dis_max_sweeps = 0;
  std::vector<int> dis_ndimwin, dis_nfirstwin;
  // results
  bool have_result = false;
  double omega[4] = {0, 0, 0, 0};
  std::vector<double> centres, spreads, log, log_centres;
  int niter = 0;
  // library-mode bookkeeping: the seedname of cinput_setopt (files of cinput_reader,
  // coverlaps, cchkpt), the options it consumed (cinput_reader adds the .win keywords
  // to them), the optional projections buffer of cset_a_matrix, exclude_bands for the
  // checkpoint, and a rejected k-point distribution (reported by the next work call)
  std::string seedname;
  std::map<std::string, Opt> applied_opts;
  double* a_matrix = nullptr;
  std::vector<int> exclude_bands;
  std::string dist_error;
  int comm = 0;
  // engine
  std::unique_ptr<Engine> eng;
  cudaStream_t stream = nullptr;
  std::string last_error;
};

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

Handle* H(void* h) { return static_cast<Handle*>(h); }

void set_opt(void* h, const char* key, const double* v, int rows, int cols, bool is_int) {
  if (!h || !key) return;
  Opt o;
  o.v.assign(v, v + (size_t)rows * cols);
  o.rows = rows;
  o.cols = cols;
  o.is_int = is_int;
  H(h)->opts[lower(key)] = o;
}

bool get_num(const Handle* h, const char* k, double& out) {
  auto it = h->opts.find(k);
  if (it == h->opts.end() || it->second.v.empty()) return false;
  out = it->second.v[0];
  return true;
}

// Fortran Ew.d edit descriptor (mantissa in [0.1, 1))
std::string fort_e(double v, int w, int d) {
  char buf[64];
  if (v == 0.0 || !std::isfinite(v)) {
    if (!std::isfinite(v)) {
      std::snprintf(buf, sizeof buf, "%*s", w, "NaN");
      return buf;
    }
    std::string m = "0." + std::string(d, '0') + "E+00";
    std::snprintf(buf, sizeof buf, "%*s", w, m.c_str());
    return buf;
  }
  const double a = std::fabs(v);
  int e = (int)std::floor(std::log10(a)) + 1;
  double mant = a / std::pow(10.0, e);
  double scale = std::pow(10.0, d);
  double r = std::round(mant * scale) / scale;
  if (r >= 1.0) {
    e += 1;
    r = std::round(a / std::pow(10.0, e) * scale) / scale;
  } else if (r < 0.1) {
    e -= 1;
    r = std::round(a / std::pow(10.0, e) * scale) / scale;
  }
  char mbuf[48];
  std::snprintf(mbuf, sizeof mbuf, "%.*f", d, r);
  char out[64];
  std::snprintf(out, sizeof out, "%s%sE%c%02d", v < 0 ? "-" : "", mbuf, e < 0 ? '-' : '+', std::abs(e));
  std::snprintf(buf, sizeof buf, "%*s", w, out);
  return buf;
}

void print_centres(const Handle* h, const double* cen4) {
  const int W = h->num_wann;
  double sx = 0, sy = 0, sz = 0, ss = 0;
  for (int n = 0; n < W; ++n) {
    std::printf("  WF centre and spread%5d  (%10.6f,%10.6f,%10.6f )%15.8f\n", n + 1, cen4[n], cen4[W + n],
                cen4[2 * W + n], cen4[3 * W + n]);
    sx += cen4[n];
    sy += cen4[W + n];
    sz += cen4[2 * W + n];
    ss += cen4[3 * W + n];
  }
  std::printf("  Sum of centres and spreads (%10.6f,%10.6f,%10.6f )%15.8f\n\n", sx, sy, sz, ss);
}

// .wout blocks of wann_main (src/wannierise.F90:451-545, :704-756, :838-880)
void print_wout(const Handle* h, const w90g::ProblemResult& r) {
  const int W = h->num_wann;
  const int rows = (int)(r.log.size() / w90g::kLogStride);
  std::printf("\n *------------------------------- WANNIERISE ---------------------------------*\n");
  std::printf(" +--------------------------------------------------------------------+<-- CONV\n");
  std::printf(" | Iter  Delta Spread     RMS Gradient      Spread (Ang^2)      Time  |<-- CONV\n");
  std::printf(" +--------------------------------------------------------------------+<-- CONV\n\n");
  const double t0 = r.log.empty() ? 0.0 : r.log[8];
  for (int i = 0; i < rows; ++i) {
    const double* lg = &r.log[(size_t)i * w90g::kLogStride];
    const int it = (int)lg[0];
    const bool lprint = (it == 0) || (it % h->num_print_cycles == 0) || it == 1 || it == h->ctl.num_iter ||
                        i == rows - 1;
    if (!lprint) continue;
    if (it == 0) {
      std::printf(" %s\n", std::string(78, '-').c_str());
      std::printf(" Initial State\n");
    } else {
      std::printf(" Cycle: %6d\n", it);
    }
    print_centres(h, &r.log_centres[(size_t)i * 4 * W]);
    const double tsec = (lg[8] - t0) * 1e-9;
    std::printf(" %6d  %s  %15.10f  %18.10f   %8.2f  <-- CONV\n", it, fort_e(lg[1], 12, 3).c_str(), lg[2], lg[3],
                tsec);
    const double* pv = it > 0 ? &r.log[(size_t)(i - 1) * w90g::kLogStride] : nullptr;
    if (h->slwf_num > 0) {
      // O_IOD = Omega_IOD + Omega_nu; its Delta holds Omega_nu fixed (src/wannierise.F90:712-740)
      if (it == 0) {
        std::printf("       O_D=%15.7f O_IOD=%15.7f O_TOT=%15.7f <-- SPRD\n", lg[4], lg[5], lg[3]);
      } else {
        std::printf("       O_IOD=%15.7f O_D=%15.7f O_TOT=%15.7f <-- SPRD\n", lg[5], lg[4], lg[3]);
        std::printf("Delta: O_IOD=%s O_D=%s O_TOT=%s <-- DLTA\n",
                    fort_e((lg[5] - lg[9]) - (pv[5] - pv[9]), 15, 7).c_str(), fort_e(lg[4] - pv[4], 15, 7).c_str(),
                    fort_e(lg[3] - pv[3], 15, 7).c_str());
      }
    } else {
      std::printf("        O_D=%15.7f O_OD=%15.7f O_TOT=%15.7f <-- SPRD\n", lg[4], lg[5], lg[3]);
      if (it > 0)
        std::printf(" Delta: O_D=%s O_OD=%s O_TOT=%s <-- DLTA\n", fort_e(lg[4] - pv[4], 15, 7).c_str(),
                    fort_e(lg[5] - pv[5], 15, 7).c_str(), fort_e(lg[3] - pv[3], 15, 7).c_str());
    }
    std::printf(" %s\n", std::string(78, '-').c_str());
  }
  if (r.converged) {
    std::printf("\n             <<<     Delta <%s  over %2d iterations     >>>\n",
                fort_e(h->ctl.conv_tol, 10, 3).c_str(), h->ctl.conv_window);
    std::printf("             <<< Wannierisation convergence criteria satisfied >>>\n\n");
  }
  std::printf(" Final State\n");
  std::vector<double> cen4(4 * W);
  for (int n = 0; n < W; ++n) {
    for (int i = 0; i < 3; ++i) cen4[i * W + n] = r.centres[n * 3 + i];
    cen4[3 * W + n] = r.spreads[n];
  }
  print_centres(h, cen4.data());
  if (h->slwf_num > 0) {
    // src/wannierise.F90:827-865
    double ssum = 0.0, pen = 0.0;
    for (int n = 0; n < W; ++n) ssum += r.spreads[n];
    const bool constrained = !h->slwf_c.empty();
    if (constrained)
      for (int n = 0; n < h->slwf_num; ++n)
        for (int i = 0; i < 3; ++i) {
          const double dx = r.centres[n * 3 + i] - h->slwf_c[(size_t)i * W + n];
          pen += dx * dx;
        }
    if (constrained) {
      std::printf("         Spreads (Ang^2)       Omega IOD_C   = %15.9f\n", r.spread.om_od);
      std::printf("        ================       Omega D       = %15.9f\n", r.spread.om_d);
      std::printf("                               Omega Rest    = %15.9f\n", ssum + r.spread.om_tot);
      std::printf("                               Penalty func  = %15.9f\n", pen);
      std::printf("    Final Spread (Ang^2)       Omega Total_C = %15.9f\n", r.spread.om_tot);
    } else {
      std::printf("         Spreads (Ang^2)       Omega IOD    = %15.9f\n", r.spread.om_od);
      std::printf("        ================       Omega D      = %15.9f\n", r.spread.om_d);
      std::printf("                               Omega Rest   = %15.9f\n", ssum + r.spread.om_tot);
      std::printf("    Final Spread (Ang^2)       Omega Total  = %15.9f\n", r.spread.om_tot);
    }
  } else {
    std::printf("         Spreads (Ang^2)       Omega I      = %15.9f\n", r.spread.om_i);
    std::printf("        ================       Omega D      = %15.9f\n", r.spread.om_d);
    std::printf("                               Omega OD     = %15.9f\n", r.spread.om_od);
    std::printf("    Final Spread (Ang^2)       Omega Total  = %15.9f\n", r.spread.om_tot);
  }
  std::printf(" %s\n", std::string(78, '-').c_str());
  std::fflush(stdout);
}

int fail(Handle* h, int code, const std::string& msg) {
  h->last_error = msg;
  if (h->iprint > 0 || code > 0) std::fprintf(stderr, "Exiting....... \n%s\n", msg.c_str());
  return code;
}

// ---- .win keywords -> options (cinput_reader / cinput_reader_special) ----------------
// How the engine reads each keyword it uses; keywords it does not use are accepted
// (read_win checks them against the reference's set) and left alone.
const char* const kWinInts[] = {"num_wann", "num_bands", "num_iter", "num_cg_steps", "conv_window",
                                "search_shells", "iprint", "num_print_cycles", "conv_noise_num", "dis_num_iter",
                                "dis_conv_window", "dis_spheres_num", "slwf_num", "num_no_guide_iter",
                                "num_guide_cycles", "optimisation", "timing_level", "num_dump_cycles"};
const char* const kWinReals[] = {"conv_tol", "trial_step", "fixed_step", "conv_noise_amp", "kmesh_tol",
                                 "dis_win_min", "dis_win_max", "dis_froz_min", "dis_froz_max", "dis_mix_ratio",
                                 "dis_conv_tol", "slwf_lambda", "symmetrize_eps", "ws_distance_tol"};
const char* const kWinLogicals[] = {"precond", "guiding_centres", "gamma_only", "slwf_constrain",
                                    "site_symmetry"};

bool in_list(const std::string& k, const char* const* list, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (k == list[i]) return true;
  return false;
}

Opt make_opt(const std::vector<double>& v, int rows, int cols, bool is_int) {
  Opt o;
  o.v = v;
  o.rows = rows;
  o.cols = cols;
  o.is_int = is_int;
  return o;
}

// Options of a tokenized .win, as cset_option_* would set them.  Returns 0 or 5 (err).
int win_options(const w90g::WinFile& w, std::map<std::string, Opt>& out, std::string& err) {
  out.clear();
  for (const auto& kv : w.keys) {
    const std::string& k = kv.first;
    const std::string& t = kv.second;
    const bool engine_int = k.compare(0, 4, "gpu_") == 0;
    if (engine_int || in_list(k, kWinInts, sizeof kWinInts / sizeof *kWinInts)) {
      int x;
      if (!w90g::parse_int(t, x)) {
        err = "Error: Problem reading keyword " + k;
        return 5;
      }
      out[k] = make_opt({(double)x}, 1, 1, true);
    } else if (in_list(k, kWinReals, sizeof kWinReals / sizeof *kWinReals)) {
      double x;
      if (!w90g::parse_real(t, x)) {
        err = "Error: Problem reading keyword " + k;
        return 5;
      }
      out[k] = make_opt({x}, 1, 1, false);
    } else if (in_list(k, kWinLogicals, sizeof kWinLogicals / sizeof *kWinLogicals)) {
      bool b;
      if (!w90g::parse_logical(t, b)) {
        err = "Error: Problem reading logical keyword " + k;
        return 5;
      }
      out[k] = make_opt({b ? 1.0 : 0.0}, 1, 1, true);
    } else if (k == "mp_grid" || k == "ws_search_size") {
      std::vector<double> x;
      if (!w90g::parse_reals(t, x) || (k == "mp_grid" && x.size() != 3)) {
        err = "Error: Problem reading keyword " + k;
        return 5;
      }
      out[k] = make_opt(x, 1, (int)x.size(), true);
    } else if (k == "exclude_bands") {
      std::vector<int> r;
      if (!w90g::parse_range_vector(t, r)) {
        err = "Error: Problem reading keyword exclude_bands";
        return 5;
      }
      out[k] = make_opt(std::vector<double>(r.begin(), r.end()), 1, (int)r.size(), true);
    }
  }
  auto cell = w.blocks.find("unit_cell_cart");
  if (cell != w.blocks.end()) {
    std::vector<std::string> rows = cell->second;
    double scale = 1.0;
    if (!rows.empty() && (rows[0].compare(0, 4, "bohr") == 0 || rows[0].compare(0, 3, "ang") == 0)) {
      if (rows[0].compare(0, 4, "bohr") == 0) scale = w90g::kBohrAngstrom;
      rows.erase(rows.begin());
    }
    std::vector<double> a;
    for (const auto& r : rows) {
      std::vector<double> x;
      if (!w90g::parse_reals(r, x) || x.size() < 3) {
        err = "Error: Problem reading block keyword unit_cell_cart";
        return 5;
      }
      for (int i = 0; i < 3; ++i) a.push_back(x[i] * scale);
    }
    if (a.size() != 9) {
      err = "Error: Wrong number of lines in block unit_cell_cart";
      return 5;
    }
    out["unit_cell_cart"] = make_opt(a, 3, 3, false);
  }
  auto kp = w.blocks.find("kpoints");
  if (kp != w.blocks.end()) {
    std::vector<double> a;
    for (const auto& r : kp->second) {
      std::vector<double> x;
      if (!w90g::parse_reals(r, x) || x.size() < 3) {
        err = "Error: Problem reading block keyword kpoints";
        return 5;
      }
      for (int i = 0; i < 3; ++i) a.push_back(x[i]);
    }
    out["kpoints"] = make_opt(a, (int)a.size() / 3, 3, false);
  }
  return 0;
}

bool same_values(const Opt& a, const Opt& b) {
  if (a.v.size() != b.v.size()) return false;
  for (size_t i = 0; i < a.v.size(); ++i)
    if (std::fabs(a.v[i] - b.v[i]) > 1e-10 * std::max(1.0, std::fabs(a.v[i]))) return false;
  return true;
}

// the k-point distribution a single-GPU engine can honour: every k on rank 0
int check_distribution(Handle* h) {
  if (!h->dist_error.empty()) return fail(h, 5, h->dist_error);
  return 0;
}

int build_spec(Handle* h, ProblemSpec& s) {
  s.W = h->num_wann;
  s.K = h->num_kpts;
  s.B = h->km.nntot;
  s.wbtot = h->km.wbtot;
  s.nnlist = h->km.nnlist;
  s.bk = h->km.bk;
  s.wb = h->km.wb;
  s.ctl = h->ctl;
  s.tensor = h->gpu_tensor;
  s.tensor_exp = h->gpu_tensor_exp;
  s.mupdate_pipe = h->gpu_mupdate_pipe;
  s.exp_smem = h->gpu_exp_smem;
  s.guiding = h->guiding;
  s.no_guide_iter = h->no_guide_iter;
  s.guide_cycles = h->guide_cycles;
  if (h->guiding) {
    s.rguide0 = h->rguide0;
    s.nnh = h->km.nnh;
    s.bka = h->km.bka;
    s.neigh = h->km.neigh;
  }
  s.slwf_num = h->slwf_num;
  s.slwf_lambda = h->slwf_lambda;
  s.slwf_c = h->slwf_c;
  if (h->site_symmetry && h->have_sym && h->sym_nk == h->num_kpts && h->sym_nb == h->num_bands) {
    s.sym_nir = h->sym_nir;
    s.sym_eps = h->symmetrize_eps;
    s.sym_ik = h->sym_ik;
    s.sym_moff = h->sym_moff;
    s.sym_mem = h->sym_mem;
    s.sym_goff = h->sym_goff;
    s.sym_grp = h->sym_grp;
    s.sym_d = h->sym_d;
    // after a disentanglement d(R,k) is replaced by D(R,k) (sitesym_replace_d_matrix_band,
    // src/disentangle.F90:237); with isolated bands the two have the same size
    s.sym_db = h->num_bands == h->num_wann ? h->sym_db : h->sym_d;
  }
  s.precond = h->precond;
  s.nrpts = h->nrpts;
  s.pc_kr = h->pc_kr;
  s.pc_r2 = h->pc_r2;
  s.pc_ndeg = h->pc_ndeg;
  return 0;
}

// leading dimension of the caller's M blocks for Engine::load/store: m_matrix_local is
// (num_bands, num_bands, nntot, num_kpts) and wann_main works on the top-left
// num_wann x num_wann of each block (src/wannierise.F90:1742-1746); 0 = packed
int mld(const Handle* h) { return h->num_bands > h->num_wann ? h->num_bands : 0; }

Engine* engine(Handle* h) {
  if (!h->eng) h->eng.reset(new Engine());
  h->eng->set_stream(h->stream);
  return h->eng.get();
}

// site_symmetry = T without its data: the reference stops reading the .dmn file
bool sym_missing(Handle* h) {
  return h->site_symmetry && !(h->have_sym && h->sym_nk == h->num_kpts && h->sym_nb == h->num_bands);
}
const char* kSymMissing = "site_symmetry = T needs the symmetry data of the .dmn file (w90g_set_sitesym)";

int do_project(Handle* h, double* m, double* u, cudaMemcpyKind in, cudaMemcpyKind out) {
  if (!h->setup_complete) return fail(h, 1, "cinput_setopt must be called before cproject_overlap");
  if (check_distribution(h)) return 5;
  if (sym_missing(h)) return fail(h, 6, kSymMissing);
  if (!m) return fail(h, 1, "m_matrix_local not set for projovlp call");
  if (!u) return fail(h, 1, "u_matrix not set for projovlp call");
  // w90_project_overlap projects only when no disentanglement ran (src/library_interface.F90:449-459)
  if (h->have_disentangled) return 0;
  if (h->num_bands != h->num_wann) return fail(h, 5, "cproject_overlap: num_bands > num_wann needs cdisentangle first");
  ProblemSpec s;
  build_spec(h, s);
  std::string err;
  Engine* e = engine(h);
  int rc = e->setup({s}, err);
  if (!rc) rc = e->load(0, m, u, in, err);
  if (!rc) rc = e->project(err);
  if (!rc) rc = e->store(0, m, u, out, err);
  if (rc) return fail(h, rc, err);
  return 0;
}

// copy one solve's result into the handle (the library's wannier_data / omega fields);
// returns the ierr of the solve (non-finite spread, failed unitarity check)
int apply_result(Handle* h, const w90g::ProblemResult& r, bool print) {
  // with selective localisation wann_main leaves omega%invariant as it was
  // (src/wannierise.F90:460-470): the disentanglement's Omega_I, else 0
  h->omega[0] = h->slwf_num > 0 ? (h->have_disentangled ? h->omega_invariant : 0.0) : r.spread.om_i;
  h->omega[1] = r.spread.om_d;
  h->omega[2] = r.spread.om_od;
  h->omega[3] = r.spread.om_tot;
  h->centres = r.centres;
  h->spreads = r.spreads;
  h->log = r.log;
  h->log_centres = r.log_centres;
  h->niter = r.niter;
  h->have_result = true;
  if (print && h->iprint > 0) print_wout(h, r);
  if (r.error == 2)
    return fail(h, 1, "tensor-core kernel: a bounded wait ran out (device status 2); the kernel drained the work "
                      "it had issued and stopped the solve");
  if (r.error) return fail(h, 1, "non-finite spread in the engine");
  if (!(r.unitarity_err <= 1e-5)) return fail(h, 1, "wann_check_unitarity: unitariety of final U violated");
  return 0;
}

int do_wannierise(Handle* h, double* m, double* u, cudaMemcpyKind in, cudaMemcpyKind out) {
  if (!h->setup_complete) return fail(h, 1, "cinput_setopt must be called before cwannierise");
  if (check_distribution(h)) return 5;
  if (sym_missing(h)) return fail(h, 6, kSymMissing);
  if (!m) return fail(h, 1, "m_matrix_local not set for wannierise");
  if (!u) return fail(h, 1, "u_matrix not set for wannierise");
  const int ldm = mld(h);
  ProblemSpec s;
  build_spec(h, s);
  std::string err;
  Engine* e = engine(h);
  int rc = e->setup({s}, err);
  if (!rc) rc = e->load(0, m, u, in, err, ldm);
  if (!rc) rc = e->wannierise(err);
  if (!rc) rc = e->store(0, m, u, out, err, ldm);
  if (rc) return fail(h, rc, err);
  return apply_result(h, e->result(0), true);
}

// w90_disentangle (src/library_interface.F90:362-420): dis_main + setup_m_loc.  Inputs:
// m (num_bands, num_bands, nntot, num_kpts), uopt = the projections
// (num_bands, num_wann, num_kpts), eig (num_bands, num_kpts).  Outputs: uopt = the
// optimal subspace (rows of the outer window, from the first), u = internal_find_u,
// m's top-left num_wann x num_wann blocks = U^H U_opt^H M U_opt' U'.
int do_disentangle(Handle* h, double* m, double* uopt, double* u, const double* eig, bool device, double* prof_ms,
                   int* prof_counts) {
  if (!h->setup_complete) return fail(h, 1, "cinput_setopt must be called before cdisentangle");
  if (check_distribution(h)) return 5;
  if (!m) return fail(h, 1, "m_matrix_local not associated for disentangle call");
  if (!u) return fail(h, 1, "u_matrix not associated for disentangle call");
  if (!uopt) return fail(h, 1, "u_opt not associated for disentangle call");
  if (!eig) return fail(h, 1, "eigval not associated for disentangle call");
  if (sym_missing(h)) return fail(h, 6, kSymMissing);
  const int W = h->num_wann;
  w90g::DisSpec ds;
  ds.nb = h->num_bands;
  ds.W = W;
  ds.K = h->num_kpts;
  ds.B = h->km.nntot;
  ds.wbtot = h->km.wbtot;
  ds.nnlist = h->km.nnlist;
  ds.wb = h->km.wb;
  ds.eig = eig;
  ds.M = m;
  ds.A = uopt;
  ds.uopt_out = uopt;
  ds.u_out = u;
  ds.m_out = m;
  ds.device = device;
  ds.stream = h->stream;
  ds.ctl = h->dis_ctl;
  ds.prof_ms = prof_ms;
  ds.prof_counts = prof_counts;
  if (h->site_symmetry) {
    ds.sym_nir = h->sym_nir;
    ds.sym_nsym = h->sym_nsym;
    ds.sym_eps = h->symmetrize_eps;
    ds.sym_ik = h->sym_ik;
    ds.sym_moff = h->sym_moff;
    ds.sym_mem = h->sym_mem;
    ds.sym_goff = h->sym_goff;
    ds.sym_grp = h->sym_grp;
    ds.sym_d = h->sym_d;
    ds.sym_db = h->sym_db;
  }
  w90g::DisResult r;
  std::string err;
  const int rc = w90g::dis_run(ds, r, err);
  h->dis_launches = r.launches;   // kernels of the last disentanglement
  if (rc) return fail(h, rc, err);
  h->omega_invariant = r.omega_invariant;
  h->dis_converged = r.converged;
  h->dis_log = r.log;
  h->dis_max_sweeps = r.max_sweeps;
  h->dis_ndimwin = r.ndimwin;
  h->dis_nfirstwin = r.nfirstwin;
  h->have_disentangled = true;
  if (h->iprint > 0) {
    const char* bar = "+---------------------------------------------------------------------+<-- DIS";
    std::printf(" %s\n |  Iter     Omega_I(i-1)      Omega_I(i)      Delta (frac.)    Time   |<-- DIS\n %s\n", bar,
                bar);
    for (size_t i = 0; i + w90g::kDisLogStride <= r.log.size(); i += w90g::kDisLogStride)
      std::printf("  %6d   %14.8f   %14.8f      %10.3E  %8.2f    <-- DIS\n", (int)r.log[i], r.log[i + 1], r.log[i + 2],
                  r.log[i + 3], r.log[i + 4]);
    std::printf("\n        Final Omega_I %14.8f (Ang^2)\n\n", r.omega_invariant);
    std::fflush(stdout);
  }
  return 0;
}

// ----------------------------------------------------------------------------
// Serving loop (continuous batching).  Jobs are admitted first-in first-out while the
// device bytes of the running jobs stay within the HBM budget and a slot is free; each
// admitted job gets its own engine on its slot's stream, so the kernels of all running
// jobs overlap on the GPU.  One worker thread keeps two chunks of graph replays in
// flight per job and polls each chunk's "all done" word through a pinned host flag and
// an event; a finished job is rotated back into the caller's buffers, its results are
// written to its handle, and its memory and slot go to the next job in the queue.
// ----------------------------------------------------------------------------
struct ServeJob {
  long long tag = 0;
  Handle* h = nullptr;
  double* d_m = nullptr;
  double* d_u = nullptr;
  ProblemSpec spec;
  size_t bytes = 0;
  double t_submit = 0.0, t_admit = 0.0;
  int slot = -1;
  std::unique_ptr<Engine> eng;
  int inflight = 0;   // chunks in flight (0..2)
  int head = 0;       // flag/event index (0/1) of the oldest chunk in flight
};

struct ServeDone {
  long long tag;
  int ierr;
  double t_submit, t_admit, t_done;
};

struct Server {
  size_t budget = 0;
  int max_active = 0, chunk = 8, device = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::unique_ptr<ServeJob>> queue;   // guarded by mu
  std::vector<ServeDone> done;                   // guarded by mu
  int pending = 0;                               // queued + running, guarded by mu
  bool stop = false;                             // guarded by mu
  std::vector<std::unique_ptr<ServeJob>> active; // worker thread only
  size_t used = 0;                               // worker thread only
  std::vector<int> free_slots;                   // worker thread only
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;               // 2 per slot
  int* d_flags = nullptr;                        // 2 per slot
  int* h_flags = nullptr;                        // pinned, 2 per slot
  std::thread worker;
  std::chrono::steady_clock::time_point t0;
  // statistics
  int peak_active = 0;
  size_t peak_bytes = 0;
  long long jobs_done = 0, iters_done = 0;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  void finish_job(ServeJob& j, int ierr) {
    std::lock_guard<std::mutex> lk(mu);
    done.push_back({j.tag, ierr, j.t_submit, j.t_admit, now()});
    --pending;
    ++jobs_done;
    cv.notify_all();
  }
  void start(ServeJob& j) {
    std::string err;
    j.eng.reset(new Engine());
    j.eng->set_stream(streams[j.slot]);
    j.eng->set_async_alloc(true);
    int rc = j.eng->setup({j.spec}, err);
    if (!rc) rc = j.eng->load(0, j.d_m, j.d_u, cudaMemcpyDeviceToDevice, err, mld(j.h));
    if (!rc) rc = j.eng->begin(err);
    j.t_admit = now();
    if (rc) j.h->last_error = err;
    j.inflight = 0;
    j.head = 0;
    if (rc) {
      j.eng.reset();
      finish_job(j, fail(j.h, rc, err));
      j.h = nullptr;   // completed
    }
  }
  int launch_chunk(ServeJob& j) {
    std::string err;
    const int idx = (j.head + j.inflight) & 1;
    const int f = j.slot * 2 + idx;
    int rc = j.eng->advance(chunk, d_flags + f, err);
    if (!rc && cudaMemcpyAsync(h_flags + f, d_flags + f, sizeof(int), cudaMemcpyDeviceToHost, streams[j.slot]) != cudaSuccess) rc = 1;
    if (!rc && cudaEventRecord(events[f], streams[j.slot]) != cudaSuccess) rc = 1;
    if (rc) j.h->last_error = err.empty() ? std::string("serve: chunk launch failed") : err;
    ++j.inflight;
    return rc;
  }
  void complete(ServeJob& j) {
    std::string err;
    int rc = j.eng->finish(err);
    if (!rc) rc = j.eng->store(0, j.d_m, j.d_u, cudaMemcpyDeviceToDevice, err, mld(j.h));
    int ierr = rc ? fail(j.h, rc, err) : apply_result(j.h, j.eng->result(0), false);
    iters_done += j.eng->result(0).niter;
    j.eng.reset();   // arena freed stream-ordered on the slot's stream
    finish_job(j, ierr);
  }
  void run() {
    cudaSetDevice(device);
    for (;;) {
      bool progress = false;
      std::vector<std::unique_ptr<ServeJob>> admit;
      {
        std::unique_lock<std::mutex> lk(mu);
        while (!queue.empty() && !free_slots.empty() && used + queue.front()->bytes <= budget) {
          std::unique_ptr<ServeJob> j = std::move(queue.front());
          queue.pop_front();
          j->slot = free_slots.back();
          free_slots.pop_back();
          used += j->bytes;
          admit.push_back(std::move(j));
        }
        if (stop && queue.empty() && active.empty() && admit.empty()) break;
      }
      for (auto& j : admit) {
        progress = true;
        start(*j);
        if (!j->h) {   // failed at start
          used -= j->bytes;
          free_slots.push_back(j->slot);
          continue;
        }
        active.push_back(std::move(j));
      }
      peak_active = std::max(peak_active, (int)active.size());
      peak_bytes = std::max(peak_bytes, used);
      for (size_t i = 0; i < active.size();) {
        ServeJob& j = *active[i];
        bool failed = false;
        while (j.inflight < 2 && j.eng->launched_iters() < j.eng->max_iter() && !failed) failed = launch_chunk(j) != 0;
        bool finished = failed;
        if (!failed && j.inflight > 0) {
          const int f = j.slot * 2 + j.head;
          const cudaError_t q = cudaEventQuery(events[f]);
          if (q == cudaSuccess) {
            progress = true;
            --j.inflight;
            j.head ^= 1;
            if (h_flags[f]) finished = true;
          } else if (q != cudaErrorNotReady) {
            j.h->last_error = std::string("serve: ") + cudaGetErrorString(q);
            failed = finished = true;
          }
        } else if (!failed) {
          finished = true;   // every iteration launched and retired
        }
        if (finished) {
          // drain the other chunk still in flight (a no-op replay) before rotating back
          cudaStreamSynchronize(streams[j.slot]);
          if (failed) {
            j.eng.reset();
            finish_job(j, fail(j.h, 1, j.h->last_error));
          } else {
            complete(j);
          }
          used -= j.bytes;
          free_slots.push_back(j.slot);
          active.erase(active.begin() + (long)i);
          progress = true;
          continue;
        }
        ++i;
      }
      if (!progress) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait_for(lk, std::chrono::microseconds(20));
      }
    }
  }
};

Server* SV(void* s) { return static_cast<Server*>(s); }

}  // namespace

extern "C" {

void* w90_create(void) { return new Handle(); }

void w90_delete(void* h) { delete H(h); }

void cset_option_int(void* h, const char* key, int value) {
  double v = value;
  set_opt(h, key, &v, 1, 1, true);
}

void cset_option_int3(void* h, const char* key, const int* value3) {
  double v[3] = {(double)value3[0], (double)value3[1], (double)value3[2]};
  set_opt(h, key, v, 1, 3, true);
}

void cset_option_intx(void* h, const char* key, const int* values, int count) {
  std::vector<double> v(values, values + count);
  set_opt(h, key, v.data(), 1, count, true);
}

void cset_option_float(void* h, const char* key, double value) { set_opt(h, key, &value, 1, 1, false); }

void cset_option_float33(void* h, const char* key, const double* value33) {
  set_opt(h, key, value33, 3, 3, false);
}

void cset_option_floatxy(void* h, const char* key, const double* values, int x, int y) {
  set_opt(h, key, values, x, y, false);
}

// w90_input_setopt (src/library_interface.F90:161-292) restricted to what wann_main uses;
// keyword defaults of src/wannier90_types.F90:170-192 and src/wannier90_readwrite.F90:647-754.
void cinput_setopt(void* hv, const char* seedname, int* ierr, int comm) {
  Handle* h = H(hv);
  *ierr = 0;
  if (!h) {
    *ierr = 1;
    return;
  }
  if (h->opts.empty()) {
    *ierr = fail(h, 1, " input_setopt called with no input");
    return;
  }
  h->seedname = seedname ? seedname : "";
  h->comm = comm;
  h->applied_opts = h->opts;
  h->exclude_bands.clear();
  {
    auto eit = h->opts.find("exclude_bands");
    if (eit != h->opts.end())
      for (double x : eit->second.v) h->exclude_bands.push_back((int)x);
  }
  double v;
  h->num_wann = get_num(h, "num_wann", v) ? (int)v : 0;
  if (h->num_wann <= 0) {
    *ierr = fail(h, 5, "Error: num_wann must be greater than zero");
    return;
  }
  h->num_bands = get_num(h, "num_bands", v) ? (int)v : h->num_wann;
  if (h->num_bands < h->num_wann) {
    *ierr = fail(h, 5, "Error: num_bands must be greater than or equal to num_wann");
    return;
  }
  auto kit = h->opts.find("kpoints");
  if (kit == h->opts.end() || kit->second.cols != 3) {
    *ierr = fail(h, 5, "Error: Did not find the kpoint information in the input file");
    return;
  }
  h->kpt_latt = kit->second.v;
  h->num_kpts = kit->second.rows;
  if (get_num(h, "num_kpts", v) && (int)v != h->num_kpts) {
    *ierr = fail(h, 5, "Error: num_kpts does not match the number of kpoints given");
    return;
  }
  auto cit = h->opts.find("unit_cell_cart");
  if (cit == h->opts.end() || cit->second.v.size() != 9) {
    *ierr = fail(h, 5, "Error: Did not find the cell information in the input file");
    return;
  }
  std::memcpy(h->real_lattice, cit->second.v.data(), 9 * sizeof(double));
  auto mit = h->opts.find("mp_grid");
  if (mit != h->opts.end() && mit->second.v.size() == 3)
    for (int i = 0; i < 3; ++i) h->mp_grid[i] = (int)mit->second.v[i];
  Control& c = h->ctl;
  c.num_iter = get_num(h, "num_iter", v) ? (int)v : 100;
  c.num_cg_steps = get_num(h, "num_cg_steps", v) ? (int)v : 5;
  c.conv_tol = get_num(h, "conv_tol", v) ? v : 1.0e-10;
  c.conv_noise_amp = get_num(h, "conv_noise_amp", v) ? v : -1.0;
  c.conv_window = (c.conv_noise_amp > 0.0) ? 5 : -1;
  if (get_num(h, "conv_window", v)) c.conv_window = (int)v;
  c.conv_noise_num = get_num(h, "conv_noise_num", v) ? (int)v : 3;
  c.fixed_step = -999.0;
  c.lfixstep = 0;
  if (get_num(h, "fixed_step", v)) {
    if (v < 0.0) {
      *ierr = fail(h, 5, "Error: fixed_step must be > 0");
      return;
    }
    c.fixed_step = v;
    if (v > 0.0) c.lfixstep = 1;
  }
  c.trial_step = 2.0;
  if (get_num(h, "trial_step", v)) {
    if (c.lfixstep) {
      *ierr = fail(h, 5, "Error: cannot specify both fixed_step and trial_step");
      return;
    }
    c.trial_step = v;
  }
  if (c.num_iter < 0 || c.num_cg_steps < 0 || c.conv_tol < 0.0 || c.conv_noise_num < 0) {
    *ierr = fail(h, 5, "Error: wannierise keyword out of range");
    return;
  }
  h->iprint = get_num(h, "iprint", v) ? (int)v : 1;
  h->num_print_cycles = get_num(h, "num_print_cycles", v) ? std::max(1, (int)v) : 1;
  h->timing_level = get_num(h, "timing_level", v) ? (int)v : 1;
  h->search_shells = get_num(h, "search_shells", v) ? (int)v : 36;
  h->kmesh_tol = get_num(h, "kmesh_tol", v) ? v : 1.0e-6;
  // engine key: gpu_tensor = 1 computes M(k,b) = U^H M0 U' on tensor cores (W <= 128)
  h->gpu_tensor = get_num(h, "gpu_tensor", v) ? (int)v : 0;
  // with gpu_tensor: gpu_tensor_exp = 1 (default) also runs exp(s D) and U dU on tensor cores
  h->gpu_tensor_exp = get_num(h, "gpu_tensor_exp", v) ? (int)v : 1;
  // with gpu_tensor and num_wann <= 32: gpu_mupdate_pipe = 1 (default) runs the M update
  // as the pipelined warp-specialised kernel, 0 as the one-CTA-per-group kernel (same digits,
  // bitwise the same result)
  h->gpu_mupdate_pipe = get_num(h, "gpu_mupdate_pipe", v) ? (int)v : 1;
  // with the tensor exp and 16 < num_wann <= 32: gpu_exp_smem = 1 keeps the exp chain's six
  // FP64 matrices in shared memory (one CTA per SM) instead of L2 (two CTAs per SM)
  h->gpu_exp_smem = get_num(h, "gpu_exp_smem", v) ? (int)v : 0;
  // options on wann_main's code path that the engine does not implement
  const char* unsupported[] = {"gamma_only", "dis_spheres_num"};
  for (const char* k : unsupported) {
    if (get_num(h, k, v)) {
      const bool active = v != 0.0;
      if (active) {
        *ierr = fail(h, 5, std::string("Option '") + k + "' is not supported by the GPU engine");
        return;
      }
    }
  }
  if (c.conv_noise_amp > 0.0) {
    *ierr = fail(h, 5, "Option 'conv_noise_amp' > 0 is not supported by the GPU engine");
    return;
  }
  std::string err;
  int rc = w90g::kmesh_get(h->real_lattice, h->kpt_latt.data(), h->num_kpts, h->search_shells, h->kmesh_tol,
                           h->km, err);
  if (rc) {
    *ierr = fail(h, rc, err);
    return;
  }
  h->guiding = get_num(h, "guiding_centres", v) ? (v != 0.0) : 0;
  h->no_guide_iter = get_num(h, "num_no_guide_iter", v) ? (int)v : 0;
  h->guide_cycles = get_num(h, "num_guide_cycles", v) ? (int)v : 1;
  h->rguide0.clear();
  if (h->guiding) {
    if (h->no_guide_iter < 0 || h->guide_cycles < 0) {
      *ierr = fail(h, 5, "Error: num_no_guide_iter and num_guide_cycles must be >= 0");
      return;
    }
    auto git = h->opts.find("guiding_centres_frac");
    if (git == h->opts.end() || git->second.cols != 3 || git->second.rows < h->num_wann) {
      *ierr = fail(h, 5, "Error: guiding_centres = T needs the projection centres (guiding_centres_frac, num_wann x 3)");
      return;
    }
    const int W = h->num_wann;
    h->rguide0.assign((size_t)3 * W, 0.0);
    for (int n = 0; n < W; ++n)
      for (int j = 0; j < 3; ++j) {
        // utility_frac_to_cart: r = sum_i frac_i a_i
        double x = 0.0;
        for (int i = 0; i < 3; ++i) x += git->second.v[(size_t)n * 3 + i] * h->real_lattice[i * 3 + j];
        h->rguide0[(size_t)j * W + n] = x;
      }
  }
  // symmetry-adapted mode (src/wannier90_readwrite.F90:387-412); the engine runs it for
  // isolated bands (the disentanglement's symmetrised Z matrices are not built)
  h->site_symmetry = get_num(h, "site_symmetry", v) ? (v != 0.0) : 0;
  h->symmetrize_eps = get_num(h, "symmetrize_eps", v) ? v : 1.0e-3;
  // selective localisation and constrained centres
  // (src/wannier90_readwrite.F90:757-802, :1660-1708; src/readwrite.F90:3266-3357)
  {
    h->slwf_num = 0;
    h->slwf_lambda = 0.0;
    h->slwf_c.clear();
    const int W = h->num_wann;
    int snum = W;
    if (get_num(h, "slwf_num", v)) {
      snum = (int)v;
      if (snum > W || snum < 1) {
        *ierr = fail(h, 5, "Error: slwf_num must be an integer between 1 and num_wann");
        return;
      }
    }
    const bool selective = snum < W;
    bool constrain = get_num(h, "slwf_constrain", v) && v != 0.0;
    if (constrain && !selective) {
      if (h->iprint > 0) std::printf(" No selective localisation requested. Ignoring constraints on centres\n");
      constrain = false;
    }
    double lambda = 1.0;
    if (get_num(h, "slwf_lambda", v)) {
      lambda = v;
      if (lambda < 0.0) {
        *ierr = fail(h, 5, "Error: slwf_lambda  must be positive.");
        return;
      }
    }
    if (selective) {
      h->slwf_num = snum;
      if (constrain) {
        auto cit = h->opts.find("slwf_centres_frac");
        if (cit == h->opts.end()) cit = h->opts.find("guiding_centres_frac");
        if (cit == h->opts.end()) {
          *ierr = fail(h, 5, "Error: slwf_constrain = true, but neither <slwf_centre> block  nor "
                             "<projection_block> are specified.");
          return;
        }
        if (cit->second.cols != 3 || cit->second.rows < W) {
          *ierr = fail(h, 5, "Error: slwf_centres_frac must be num_wann x 3");
          return;
        }
        h->slwf_lambda = lambda;
        h->slwf_c.assign((size_t)3 * W, 0.0);
        for (int n = 0; n < W; ++n)
          for (int j = 0; j < 3; ++j) {
            double x = 0.0;   // utility_frac_to_cart
            for (int i = 0; i < 3; ++i) x += cit->second.v[(size_t)n * 3 + i] * h->real_lattice[i * 3 + j];
            h->slwf_c[(size_t)j * W + n] = x;
          }
      }
    }
  }
  // disentanglement keywords (src/readwrite.F90:651-682, src/wannier90_readwrite.F90:824-854)
  {
    w90g::DisControl d;
    if (get_num(h, "dis_win_min", v)) d.win_min = v;
    if (get_num(h, "dis_win_max", v)) d.win_max = v;
    if (d.win_max < d.win_min) {
      *ierr = fail(h, 5, "Error: w90_readwrite_read_dis_manifold: check disentanglement windows (win_max < win_min !)");
      return;
    }
    const bool fmax = get_num(h, "dis_froz_max", v);
    if (fmax) {
      d.froz_max = v;
      d.frozen_states = true;
    }
    const bool fmin = get_num(h, "dis_froz_min", v);
    if (fmin) d.froz_min = v;
    if (fmin && !fmax) {
      *ierr = fail(h, 5, "Error: w90_readwrite_read_dis_manifold: found dis_froz_min but not dis_froz_max");
      return;
    }
    if (d.froz_max < d.froz_min) {
      *ierr = fail(h, 5, "Error: w90_readwrite_read_dis_manifold: check disentanglement frozen windows");
      return;
    }
    if (get_num(h, "dis_num_iter", v)) d.num_iter = (int)v;
    if (d.num_iter < 0) {
      *ierr = fail(h, 5, "Error: dis_num_iter must be positive");
      return;
    }
    if (get_num(h, "dis_mix_ratio", v)) d.mix_ratio = v;
    if (d.mix_ratio <= 0.0 || d.mix_ratio > 1.0) {
      *ierr = fail(h, 5, "Error: dis_mix_ratio must be greater than 0.0 but not greater than 1.0");
      return;
    }
    if (get_num(h, "dis_conv_tol", v)) d.conv_tol = v;
    if (d.conv_tol < 0.0) {
      *ierr = fail(h, 5, "Error: dis_conv_tol must be positive");
      return;
    }
    if (get_num(h, "dis_conv_window", v)) d.conv_window = (int)v;
    if (d.conv_window < 0) {
      *ierr = fail(h, 5, "Error: dis_conv_window must be positive");
      return;
    }
    h->dis_ctl = d;
    h->have_disentangled = false;
    h->dis_log.clear();
  }
  h->precond = get_num(h, "precond", v) ? (v != 0.0) : 0;
  h->nrpts = 0;
  h->pc_kr.clear();
  h->pc_r2.clear();
  h->pc_ndeg.clear();
  if (h->precond) {
    if (h->mp_grid[0] < 1 || h->mp_grid[1] < 1 || h->mp_grid[2] < 1) {
      *ierr = fail(h, 5, "Error: precond = T needs mp_grid");
      return;
    }
    int ws[3] = {2, 2, 2};   // ws_search_size default (src/types.F90:78)
    auto wit = h->opts.find("ws_search_size");
    if (wit != h->opts.end()) {
      for (int i = 0; i < 3; ++i) ws[i] = (int)wit->second.v[wit->second.v.size() == 3 ? i : 0];
    }
    const double wtol = get_num(h, "ws_distance_tol", v) ? v : 1.0e-5;
    std::vector<int> irvec, ndegen;
    rc = w90g::ws_vectors(h->real_lattice, h->mp_grid, ws, wtol, irvec, ndegen, err);
    if (rc) {
      *ierr = fail(h, rc, err);
      return;
    }
    const int NR = (int)ndegen.size(), K = h->num_kpts;
    h->nrpts = NR;
    h->pc_kr.resize((size_t)2 * K * NR);
    h->pc_r2.resize(NR);
    h->pc_ndeg.resize(NR);
    const double twopi = 6.283185307179586476925287;
    for (int r = 0; r < NR; ++r) {
      const double n[3] = {(double)irvec[3 * r], (double)irvec[3 * r + 1], (double)irvec[3 * r + 2]};
      // rvec_cart = matmul(real_lattice, irvec) exactly as the reference forms it
      // (src/wannierise.F90:1341): component i is a_i . n
      double r2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double x = h->real_lattice[i * 3] * n[0] + h->real_lattice[i * 3 + 1] * n[1] +
                         h->real_lattice[i * 3 + 2] * n[2];
        r2 += x * x;
      }
      h->pc_r2[r] = r2;
      h->pc_ndeg[r] = (double)ndegen[r];
      for (int k = 0; k < K; ++k) {
        const double* kp = &h->kpt_latt[(size_t)3 * k];
        const double rdotk = twopi * (kp[0] * n[0] + kp[1] * n[1] + kp[2] * n[2]);
        h->pc_kr[((size_t)k * NR + r) * 2] = std::cos(rdotk);
        h->pc_kr[((size_t)k * NR + r) * 2 + 1] = -std::sin(rdotk);
      }
    }
  }
  h->centres.assign(3 * h->num_wann, 0.0);
  h->spreads.assign(h->num_wann, 0.0);
  h->setup_complete = true;
  h->opts.clear();   // src/library_interface.F90:284-290 clears the settings after use
}

void cset_eigval(void* h, double* eigval) { H(h)->eigval = eigval; }
void cset_m_local(void* h, double* m) { H(h)->m_local = m; }
void cset_u_matrix(void* h, double* u) { H(h)->u_matrix = u; }
void cset_u_opt(void* h, double* u) { H(h)->u_opt = u; }

void cdisentangle(void* hv, int* ierr) {
  Handle* h = H(hv);
  // projections given through cset_a_matrix are the initial u_opt (nb x nw x nk)
  if (h->a_matrix && h->u_opt && h->setup_complete && h->a_matrix != h->u_opt)
    std::memcpy(h->u_opt, h->a_matrix, sizeof(double) * 2 * h->num_bands * h->num_wann * h->num_kpts);
  *ierr = do_disentangle(h, h->m_local, h->u_opt, h->u_matrix, h->eigval, false, nullptr, nullptr);
}

void w90g_disentangle_device(void* hv, double* d_m, double* d_uopt, double* d_u, const double* d_eig, int* ierr) {
  *ierr = do_disentangle(H(hv), d_m, d_uopt, d_u, d_eig, true, nullptr, nullptr);
}

int w90g_profile_dis_device(void* hv, double* d_m, double* d_uopt, double* d_u, const double* d_eig, double* ms,
                            int* counts) {
  for (int i = 0; i < w90g::kDisKernels; ++i) {
    ms[i] = 0.0;
    counts[i] = 0;
  }
  return do_disentangle(H(hv), d_m, d_uopt, d_u, d_eig, true, ms, counts);
}

const char* w90g_dis_kernel_name(int i) { return w90g::dis_kernel_name(i); }

void cwannierise(void* hv, int* ierr) {
  Handle* h = H(hv);
  // w90_wannierise requires u_opt as well (src/library_interface.F90:480-486)
  if (!h->u_opt) {
    *ierr = fail(h, 1, "u_opt not set for wannierise");
    return;
  }
  *ierr = do_wannierise(h, h->m_local, h->u_matrix, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
}

void cproject_overlap(void* hv, int* ierr) {
  Handle* h = H(hv);
  // projections given through cset_a_matrix are A(k) (num_bands = num_wann here)
  if (h->a_matrix && h->u_matrix && h->setup_complete && h->num_bands == h->num_wann &&
      h->a_matrix != h->u_matrix)
    std::memcpy(h->u_matrix, h->a_matrix, sizeof(double) * 2 * h->num_wann * h->num_wann * h->num_kpts);
  *ierr = do_project(h, h->m_local, h->u_matrix, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
}

void w90g_wannierise_device(void* hv, double* d_m, double* d_u, int* ierr) {
  *ierr = do_wannierise(H(hv), d_m, d_u, cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

void w90g_project_overlap_device(void* hv, double* d_m, double* d_u, int* ierr) {
  *ierr = do_project(H(hv), d_m, d_u, cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

void cget_nn(void* hv, int* nn) {
  Handle* h = H(hv);
  *nn = h->setup_complete ? h->km.nntot : 0;
}

void cget_nnkp(void* hv, int* nnkp) {
  // w90_get_nnkp: nnlist(nk, nntot), 1-based, Fortran column-major (k fastest)
  Handle* h = H(hv);
  if (!h->setup_complete) return;
  const int K = h->num_kpts, B = h->km.nntot;
  for (int b = 0; b < B; ++b)
    for (int k = 0; k < K; ++k) nnkp[b * K + k] = h->km.nnlist[(size_t)k * B + b] + 1;
}

void cget_gkpb(void* hv, int* gkpb) {
  // nncell(3, nk, nntot), Fortran column-major
  Handle* h = H(hv);
  if (!h->setup_complete) return;
  const int K = h->num_kpts, B = h->km.nntot;
  for (int b = 0; b < B; ++b)
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < 3; ++i) gkpb[(b * K + k) * 3 + i] = h->km.nncell[((size_t)k * B + b) * 3 + i];
}

void cget_centres(void* hv, double* centres) {
  Handle* h = H(hv);
  std::copy(h->centres.begin(), h->centres.end(), centres);
}

void cget_spreads(void* hv, double* spreads) {
  Handle* h = H(hv);
  std::copy(h->spreads.begin(), h->spreads.end(), spreads);
}

void cget_omega(void* hv, double* omega4) {
  Handle* h = H(hv);
  std::copy(h->omega, h->omega + 4, omega4);
}

const char* w90g_last_error(void* hv) { return H(hv)->last_error.c_str(); }

int w90g_get_dis_log(void* hv, double* rows, int max_rows) {
  Handle* h = H(hv);
  const int n = std::min(max_rows, (int)(h->dis_log.size() / w90g::kDisLogStride));
  std::copy(h->dis_log.begin(), h->dis_log.begin() + (size_t)n * w90g::kDisLogStride, rows);
  return n;
}

// sitesym_read's data (src/sitesym.F90:698-765): the .dmn counts, 1-based ik2ir(nk),
// ir2ik(nkirr), kptsym(nsym, nkirr), d_matrix_wann(nw, nw, nsym, nkirr) and
// d_matrix_band(nb, nb, nsym, nkirr), Fortran order, complex as (re, im) pairs.  The
// star / little-group tables are built here, in the reference's loop order.
int w90g_set_sitesym(void* hv, int nb, int nsym, int nkirr, int nk, const int* ik2ir, const int* ir2ik,
                     const int* kptsym, const double* d_wann, const double* d_band) {
  Handle* h = H(hv);
  if (!h->setup_complete) return fail(h, 1, "cinput_setopt must be called before w90g_set_sitesym");
  if (nb != h->num_bands) return fail(h, 6, "Error: Number of bands is not correct (sitesym_read)");
  if (nk != h->num_kpts) return fail(h, 6, "Error: Number of k-points is not correct (sitesym_read)");
  w90g::SymTables t;
  std::string msg;
  if (int rc = w90g::build_sym_tables(h->num_wann, nb, nsym, nkirr, nk, ik2ir, ir2ik, kptsym, d_wann, d_band, t, msg))
    return fail(h, rc, msg);
  h->sym_nir = t.nir;
  h->sym_nsym = t.nsym;
  h->sym_nk = nk;
  h->sym_nb = nb;
  h->sym_ik = t.ik;
  h->sym_moff = t.moff;
  h->sym_mem = t.mem;
  h->sym_goff = t.goff;
  h->sym_grp = t.grp;
  h->sym_d = t.d;
  h->sym_db = t.db;
  h->have_sym = true;
  return 0;
}

void w90g_get_dis_windows(void* hv, int* ndimwin, int* nfirstwin) {
  Handle* h = H(hv);
  std::copy(h->dis_ndimwin.begin(), h->dis_ndimwin.end(), ndimwin);
  std::copy(h->dis_nfirstwin.begin(), h->dis_nfirstwin.end(), nfirstwin);
}

void w90g_get_dis_info(void* hv, double* info4) {
  Handle* h = H(hv);
  info4[0] = h->omega_invariant;
  info4[1] = (double)h->dis_converged;
  info4[2] = (double)(h->dis_log.size() / w90g::kDisLogStride);
  info4[3] = (double)h->dis_max_sweeps;
}

int w90g_get_log(void* hv, double* rows, int max_rows) {
  Handle* h = H(hv);
  const int n = std::min(max_rows, (int)(h->log.size() / w90g::kLogStride));
  std::copy(h->log.begin(), h->log.begin() + (size_t)n * w90g::kLogStride, rows);
  return n;
}

int w90g_get_log_centres(void* hv, double* rows, int max_rows) {
  Handle* h = H(hv);
  const size_t stride = 4 * (size_t)h->num_wann;
  if (!stride) return 0;
  const int n = std::min(max_rows, (int)(h->log_centres.size() / stride));
  std::copy(h->log_centres.begin(), h->log_centres.begin() + (size_t)n * stride, rows);
  return n;
}

void w90g_set_stream(void* hv, void* cuda_stream) {
  Handle* h = H(hv);
  h->stream = (cudaStream_t)cuda_stream;
  if (h->eng) h->eng->set_stream(h->stream);
}

int w90g_profile_device(void* hv, double* d_m, double* d_u, int max_iters, double* ms, int* counts) {
  Handle* h = H(hv);
  if (!h->setup_complete) return fail(h, 1, "cinput_setopt must be called before w90g_profile_device");
  if (sym_missing(h)) return fail(h, 6, kSymMissing);
  ProblemSpec s;
  build_spec(h, s);
  std::string err;
  Engine* e = engine(h);
  int rc = e->setup({s}, err);
  if (!rc) rc = e->load(0, d_m, d_u, cudaMemcpyDeviceToDevice, err, mld(h));
  if (!rc) rc = e->wannierise_profiled(max_iters, ms, counts, err);
  if (rc) return fail(h, rc, err);
  return 0;
}

double w90g_profile_exp_products(void* hv) {
  Handle* h = H(hv);
  return h->eng ? h->eng->last_exp_products() : 0.0;
}

const char* w90g_profile_kernel_name(int i) {
  return (i >= 0 && i < w90g::kPNum) ? w90g::kProfNames[i] : "";
}

int w90g_ws_vectors(const double* real_lattice33, const int* mp_grid3, const int* search_size3,
                    double ws_distance_tol, int* irvec_out, int* ndegen_out, int max_pts) {
  std::vector<int> irvec, ndegen;
  std::string err;
  if (w90g::ws_vectors(real_lattice33, mp_grid3, search_size3, ws_distance_tol, irvec, ndegen, err)) return -1;
  const int n = (int)ndegen.size();
  if (n <= max_pts) {
    std::copy(irvec.begin(), irvec.end(), irvec_out);
    std::copy(ndegen.begin(), ndegen.end(), ndegen_out);
  }
  return n;
}

double w90g_measure_fp64_peak(void) {
  double t = 0.0;
  std::string err;
  if (w90g::measure_fp64_peak(&t, err)) return -1.0;
  return t;
}

// Batched form: independent problems (each set up on its own handle) solved together.
// Problems are grouped by the M-update variant their width selects (tensor path with
// padded width 8 / 16 / 32 / 64 / 128 when requested, FP64 path otherwise); each group
// is one engine whose iteration graph covers all of its problems, and the groups run
// concurrently on their own streams.
void w90g_wannierise_batch_device(void** handles, int nprob, double** d_m, double** d_u, int* ierr) {
  struct Group {
    std::vector<int> idx;
    std::vector<ProblemSpec> specs;
    std::unique_ptr<Engine> eng;
    cudaStream_t stream = nullptr;
    int rc = 0;
    std::string err;
  };
  std::map<int, Group> groups;   // key: 0 fp64, 8/16/32 tensor width class
  for (int i = 0; i < nprob; ++i) {
    Handle* h = H(handles[i]);
    ierr[i] = 0;
    if (!h->setup_complete || !d_m[i] || !d_u[i]) {
      ierr[i] = fail(h, 1, "batch: handle not set up or buffers missing");
      continue;
    }
    if (sym_missing(h)) {
      ierr[i] = fail(h, 6, kSymMissing);
      continue;
    }
    ProblemSpec s;
    build_spec(h, s);
    int key = 0;
    if (s.tensor && s.W <= 128) key = s.W <= 8 ? 8 : (s.W <= 16 ? 16 : (s.W <= 32 ? 32 : (s.W <= 64 ? 64 : 128)));
    if (key && key <= 32 && !s.mupdate_pipe) key += 1000;   // the one-CTA-per-group kernel
    if (key && !s.tensor_exp) key += 2000;                   // exp(s D) on the FP64 pipe
    if (key == 32 && s.tensor_exp && s.exp_smem) key += 4000;  // exp matrices in shared memory
    groups[key].idx.push_back(i);
    groups[key].specs.push_back(s);
  }
  std::vector<std::thread> threads;
  for (auto& kv : groups) {
    Group* g = &kv.second;
    threads.emplace_back([g, d_m, d_u, handles]() {
      g->eng.reset(new Engine());
      if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess) {
        g->rc = 1;
        g->err = "batch: stream creation failed";
        return;
      }
      g->eng->set_stream(g->stream);
      g->rc = g->eng->setup(g->specs, g->err);
      for (size_t j = 0; j < g->idx.size() && !g->rc; ++j)
        g->rc = g->eng->load((int)j, d_m[g->idx[j]], d_u[g->idx[j]], cudaMemcpyDeviceToDevice, g->err,
                             mld(H(handles[g->idx[j]])));
      if (!g->rc) g->rc = g->eng->wannierise(g->err);
      for (size_t j = 0; j < g->idx.size() && !g->rc; ++j)
        g->rc = g->eng->store((int)j, d_m[g->idx[j]], d_u[g->idx[j]], cudaMemcpyDeviceToDevice, g->err,
                              mld(H(handles[g->idx[j]])));
    });
  }
  for (auto& t : threads) t.join();
  for (auto& kv : groups) {
    Group& g = kv.second;
    for (size_t j = 0; j < g.idx.size(); ++j) {
      Handle* h = H(handles[g.idx[j]]);
      if (g.rc) {
        ierr[g.idx[j]] = fail(h, g.rc, g.err);
        continue;
      }
      ierr[g.idx[j]] = apply_result(h, g.eng->result((int)j), false);
    }
    g.eng.reset();
    if (g.stream) cudaStreamDestroy(g.stream);
  }
}

void* w90g_server_create(double hbm_budget_bytes, int max_active, int chunk_iters) {
  Server* sv = new Server();
  sv->budget = hbm_budget_bytes > 0 ? (size_t)hbm_budget_bytes : 0;
  sv->max_active = std::max(1, std::min(max_active, 1024));
  sv->chunk = std::max(1, chunk_iters);
  sv->t0 = std::chrono::steady_clock::now();
  cudaGetDevice(&sv->device);
  const int n = sv->max_active;
  bool ok = cudaMalloc(&sv->d_flags, (size_t)2 * n * sizeof(int)) == cudaSuccess &&
            cudaHostAlloc(&sv->h_flags, (size_t)2 * n * sizeof(int), cudaHostAllocDefault) == cudaSuccess;
  for (int i = 0; i < n && ok; ++i) {
    cudaStream_t st;
    ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) sv->streams.push_back(st);
    for (int e = 0; e < 2 && ok; ++e) {
      cudaEvent_t ev;
      ok = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
      if (ok) sv->events.push_back(ev);
    }
    sv->free_slots.push_back(n - 1 - i);
  }
  if (!ok) {
    w90g_server_delete(sv);
    return nullptr;
  }
  sv->worker = std::thread([sv]() { sv->run(); });
  return sv;
}

int w90g_server_submit(void* server, void* handle, double* d_m, double* d_u, long long tag) {
  Server* sv = SV(server);
  Handle* h = H(handle);
  if (!sv || !h) return 1;
  if (!h->setup_complete || !d_m || !d_u) return fail(h, 1, "serve: handle not set up or buffers missing");
  if (sym_missing(h)) return fail(h, 6, kSymMissing);
  std::unique_ptr<ServeJob> j(new ServeJob());
  j->tag = tag;
  j->h = h;
  j->d_m = d_m;
  j->d_u = d_u;
  build_spec(h, j->spec);
  j->bytes = Engine::estimate_bytes({j->spec});
  if (j->bytes > sv->budget) return fail(h, 2, "serve: job needs more device memory than the server's budget");
  std::lock_guard<std::mutex> lk(sv->mu);
  j->t_submit = sv->now();
  sv->queue.push_back(std::move(j));
  ++sv->pending;
  sv->cv.notify_all();
  return 0;
}

int w90g_server_poll(void* server, long long* tags, int* ierr, double* t_submit, double* t_admit, double* t_done,
                     int max) {
  Server* sv = SV(server);
  std::lock_guard<std::mutex> lk(sv->mu);
  const int n = std::min(max, (int)sv->done.size());
  for (int i = 0; i < n; ++i) {
    const ServeDone& d = sv->done[i];
    if (tags) tags[i] = d.tag;
    if (ierr) ierr[i] = d.ierr;
    if (t_submit) t_submit[i] = d.t_submit;
    if (t_admit) t_admit[i] = d.t_admit;
    if (t_done) t_done[i] = d.t_done;
  }
  sv->done.erase(sv->done.begin(), sv->done.begin() + n);
  return n;
}

int w90g_server_pending(void* server) {
  Server* sv = SV(server);
  std::lock_guard<std::mutex> lk(sv->mu);
  return sv->pending;
}

void w90g_server_drain(void* server) {
  Server* sv = SV(server);
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->cv.wait(lk, [sv]() { return sv->pending == 0; });
}

void w90g_server_stats(void* server, double* out4) {
  Server* sv = SV(server);
  std::lock_guard<std::mutex> lk(sv->mu);
  out4[0] = sv->peak_active;
  out4[1] = (double)sv->peak_bytes;
  out4[2] = (double)sv->jobs_done;
  out4[3] = (double)sv->iters_done;
}

double w90g_server_now(void* server) { return SV(server)->now(); }

void w90g_server_delete(void* server) {
  Server* sv = SV(server);
  if (!sv) return;
  if (sv->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->stop = true;
      sv->cv.notify_all();
    }
    sv->worker.join();
  }
  for (auto st : sv->streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (auto ev : sv->events) cudaEventDestroy(ev);
  if (sv->d_flags) cudaFree(sv->d_flags);
  if (sv->h_flags) cudaFreeHost(sv->h_flags);
  delete sv;
}

// ---- seed-file readers (no handle: plain arrays; err receives the message) ----------
static void put_err(const std::string& e, char* err, int errlen) {
  if (err && errlen > 0) {
    std::strncpy(err, e.c_str(), (size_t)errlen - 1);
    err[errlen - 1] = '\0';
  }
}

int w90g_read_mmn(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell, double* m,
                  int nthreads, char* err, int errlen) {
  std::string e;
  const int rc = w90g::read_mmn(path, nb, nk, nntot, nnlist, nncell, m, nthreads, e);
  put_err(e, err, errlen);
  return rc;
}

int w90g_read_amn(const char* path, int nb, int nproj, int nk, double* a, int nthreads, char* err, int errlen) {
  std::string e;
  const int rc = w90g::read_amn(path, nb, nproj, nk, a, nthreads, e);
  put_err(e, err, errlen);
  return rc;
}

int w90g_read_mmn_device(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell,
                         double* d_m, void* stream, int* used_gpu, long long* launches, double* timing3, char* err,
                         int errlen) {
  std::string e;
  int ug = 0;
  long long nl = 0;
  const int rc =
      w90g::read_mmn_device(path, nb, nk, nntot, nnlist, nncell, d_m, (cudaStream_t)stream, &ug, &nl, timing3, e);
  if (used_gpu) *used_gpu = ug;
  if (launches) *launches = nl;
  put_err(e, err, errlen);
  return rc;
}

int w90g_read_eig(const char* path, int nb, int nk, double* eig, char* err, int errlen) {
  std::string e;
  const int rc = w90g::read_eig(path, nb, nk, eig, e);
  put_err(e, err, errlen);
  return rc;
}

long long w90g_kernel_launches(void* hv) {
  Handle* h = H(hv);
  return (h->eng ? h->eng->launches() : 0) + h->dis_launches;
}


// ---- the remaining names of the reference's C++ prototypes (src/wannier90.hh:9-31) ----

// cinput_reader -> w90_input_reader (src/c_interface.F90:70-80,
// src/library_interface.F90:294-360): after cinput_setopt, the other keywords of
// seedname.win; keywords the .win sets take precedence over earlier options, the system
// (num_wann, num_bands, mp_grid, unit_cell_cart, kpoints) must agree with what
// cinput_setopt received, and the setup (k-mesh, preconditioner tables, windows) is
// redone with the merged options.
void cinput_reader(void* hv, int* ierr) {
  Handle* h = H(hv);
  *ierr = 0;
  if (!h) {
    *ierr = 1;
    return;
  }
  if (!h->opts.empty() || !h->setup_complete) {
    *ierr = fail(h, 1, "Error: input reader called when unspent options present (setopt must be called first)");
    return;
  }
  w90g::WinFile w;
  std::string err;
  int rc = w90g::read_win(h->seedname + ".win", w, err);
  std::map<std::string, Opt> win;
  if (!rc) rc = win_options(w, win, err);
  if (rc) {
    *ierr = fail(h, rc, err);
    return;
  }
  std::map<std::string, Opt> merged = h->applied_opts;
  for (const auto& kv : win) {
    const std::string& k = kv.first;
    const bool system = k == "num_wann" || k == "num_bands" || k == "mp_grid" || k == "unit_cell_cart" ||
                        k == "kpoints";
    if (system) {
      auto it = merged.find(k);
      if (it != merged.end() && !same_values(it->second, kv.second)) {
        *ierr = fail(h, 5, "Error: " + k + " of " + h->seedname +
                               ".win differs from the value set through the library");
        return;
      }
    }
    merged[k] = kv.second;
  }
  h->opts = merged;
  h->setup_complete = false;
  const std::string seed = h->seedname;
  cinput_setopt(hv, seed.c_str(), ierr, h->comm);
}

// cinput_reader_special (src/wannier90.hh:11): the whole input, system included, from
// seedname.win -- the file form of cset_option_* + cinput_setopt (wannier90.x reads it
// with w90_wannier90_readwrite_read_special, src/library_interface.F90:203-218).
void cinput_reader_special(void* hv, const char* seedname, int* ierr) {
  Handle* h = H(hv);
  *ierr = 0;
  if (!h || !seedname) {
    *ierr = 1;
    return;
  }
  if (!h->opts.empty()) {
    *ierr = fail(h, 1, "Error: (library use) options interface and .win parsing clash.  See library "
                       "documentation \"setting options.\" (readwrite.F90)");
    return;
  }
  w90g::WinFile w;
  std::string err;
  int rc = w90g::read_win(std::string(seedname) + ".win", w, err);
  std::map<std::string, Opt> win;
  if (!rc) rc = win_options(w, win, err);
  if (rc) {
    *ierr = fail(h, rc, err);
    return;
  }
  h->opts = win;
  cinput_setopt(hv, seedname, ierr, h->comm);
}

// cset_a_matrix (src/wannier90.hh:31): the caller's projections A_mn(k), complex
// (num_bands, num_wann, num_kpts).  coverlaps reads seedname.amn into it; cproject_overlap
// (isolated bands) and cdisentangle take their starting u_matrix / u_opt from it.
void cset_a_matrix(void* hv, double* a) { H(hv)->a_matrix = a; }

// cset_kpoint_distribution (src/wannier90.hh:28; set_kpoint_distribution,
// src/wannier_prog.F90:798-820): the rank owning each k-point.  One process drives one
// GPU and holds every k, so only the all-zero distribution is accepted; any other makes
// the next cproject_overlap / cdisentangle / cwannierise return 5.
void cset_kpoint_distribution(void* hv, const int* dist) {
  Handle* h = H(hv);
  h->dist_error.clear();
  if (!dist) return;
  if (!h->setup_complete) {
    h->dist_error = "Error in k-point distribution: set after cinput_setopt (num_kpts unknown)";
    return;
  }
  for (int k = 0; k < h->num_kpts; ++k)
    if (dist[k] != 0) {
      h->dist_error = "k-point distribution over several ranks is not supported by the single-GPU engine "
                      "(every k-point must be on rank 0)";
      return;
    }
}

// cset_parallel_comms (src/wannier90.hh:29): the MPI communicator, kept and not used.
void cset_parallel_comms(void* hv, int comm) { H(hv)->comm = comm; }

// coverlaps (src/wannier90.hh:21; overlaps, src/wannier_prog.F90:478-537): read
// seedname.mmn into m_matrix_local and seedname.amn into the projections -- the
// cset_a_matrix buffer if one is set, else u_matrix (isolated) / u_opt (entangled) --
// with overlap_read's checks and messages (src/overlap.F90:234-366).
void coverlaps(void* hv, int* ierr) {
  Handle* h = H(hv);
  *ierr = 0;
  if (!h->setup_complete) {
    *ierr = fail(h, 1, "kmesh is not setup before calling overlaps read routine");
    return;
  }
  if (check_distribution(h)) {
    *ierr = 5;
    return;
  }
  const bool entangled = h->num_bands > h->num_wann;
  double* a = h->a_matrix ? h->a_matrix : (entangled ? h->u_opt : h->u_matrix);
  if (!a) {
    *ierr = fail(h, 1, entangled ? "u_opt not associated at overlaps read routine"
                                 : "u_matrix not associated at overlaps read routine");
    return;
  }
  if (!h->m_local) {
    *ierr = fail(h, 1, "m_matrix_local not associated at overlaps read routine");
    return;
  }
  char err[512] = {0};
  int rc = w90g_read_mmn((h->seedname + ".mmn").c_str(), h->num_bands, h->num_kpts, h->km.nntot,
                         h->km.nnlist.data(), h->km.nncell.data(), h->m_local, 0, err, (int)sizeof err);
  if (!rc) rc = w90g_read_amn((h->seedname + ".amn").c_str(), h->num_bands, h->num_wann, h->num_kpts, a, 0, err,
                              (int)sizeof err);
  if (rc) *ierr = fail(h, rc, err);
}

// cchkpt (src/wannier90.hh:9; write_chkpt, src/wannier_prog.F90:575-700): write
// seedname.chk with the checkpoint label (e.g. "postdis", "postwann") in the layout of
// w90_wannier90_readwrite_write_chkpt (src/wannier90_readwrite.F90:2278-2373): the
// caller's u_matrix, u_opt and the leading num_wann x num_wann block of every m_matrix
// block, the centres and spreads of the last wannierisation, the windows and Omega_I of
// the last disentanglement.  Errors go to w90g_last_error (the prototype returns none).
void cchkpt(void* hv, const char* label) {
  Handle* h = H(hv);
  h->last_error.clear();
  if (!h->setup_complete) {
    fail(h, 1, "cinput_setopt must be called before write_chkpt");
    return;
  }
  if (!h->u_opt) {
    fail(h, 1, "u_opt not set for write_chkpt call");
    return;
  }
  if (!h->u_matrix) {
    fail(h, 1, "u_matrix not set for write_chkpt call");
    return;
  }
  if (!h->m_local) {
    fail(h, 1, "m_matrix_local not set for write_chkpt call");
    return;
  }
  w90g::ChkData d;
  char date[64];
  const std::time_t now = std::time(nullptr);
  std::tm tmv;
  localtime_r(&now, &tmv);
  // io_date's fields: day right-justified in 2, month abbreviation, year; hh:mm:ss
  static const char* const months[] = {"Jan", "Feb", "Mar", "Apr", "May", "Jun",
                                       "Jul", "Aug", "Sep", "Oct", "Nov", "Dec"};
  std::snprintf(date, sizeof date, "written on %2d%s%04d at %02d:%02d:%02d ", tmv.tm_mday, months[tmv.tm_mon],
                tmv.tm_year + 1900, tmv.tm_hour, tmv.tm_min, tmv.tm_sec);
  d.header = date;
  d.num_bands = h->num_bands;
  d.num_kpts = h->num_kpts;
  d.nntot = h->km.nntot;
  d.num_wann = h->num_wann;
  d.exclude_bands = h->exclude_bands;
  std::memcpy(d.real_lattice, h->real_lattice, sizeof d.real_lattice);
  for (int i = 0; i < 3; ++i) d.mp_grid[i] = h->mp_grid[i];
  d.kpt_latt = h->kpt_latt.data();
  d.checkpoint = label ? label : "postwann";
  d.have_disentangled = h->have_disentangled;
  if (h->have_disentangled) {
    d.omega_invariant = h->omega_invariant;
    d.ndimwin = h->dis_ndimwin;
    d.lwindow.assign((size_t)h->num_bands * h->num_kpts, 0);
    for (int k = 0; k < h->num_kpts; ++k)
      for (int i = 0; i < h->dis_ndimwin[k]; ++i)
        d.lwindow[(size_t)k * h->num_bands + h->dis_nfirstwin[k] + i] = 1;
  }
  d.u_opt = h->u_opt;
  d.u = h->u_matrix;
  d.m = h->m_local;
  d.ldm = h->num_bands;
  d.centres = h->centres.data();
  d.spreads = h->spreads.data();
  std::string err;
  if (w90g::write_chk(h->seedname + ".chk", d, err)) fail(h, 6, err);
}

}  // extern "C"
