// Host-side .win reader and .chk writer (see winfile.h).
#include "winfile.h"

#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <set>

#include "kmesh.h"

namespace w90g {

namespace {

// Keywords and blocks that wannier90.x or postw90.x accept: the union the reference
// scans for before it reports unrecognised keywords (src/readwrite.F90:903-1176), plus
// exclude_bands, which w90_wannier90_readwrite_read consumes itself.  A caller's .win
// must keep working, so the set is the reference's; the engine uses the wannierise,
// k-mesh and disentanglement ones and accepts the rest without acting on them.
const char* const kKeywords[] = {
    "adpt_smr", "adpt_smr_fac", "adpt_smr_max", "auto_projections", "bands_num_points", "bands_plot",
    "bands_plot_dim", "bands_plot_format", "bands_plot_mode", "bands_plot_project", "berry",
    "berry_curv_adpt_kmesh", "berry_curv_adpt_kmesh_thresh", "berry_curv_unit", "berry_kmesh",
    "berry_kmesh_spacing", "berry_task", "boltz_2d_dir", "boltz_bandshift", "boltz_bandshift_energyshift",
    "boltz_bandshift_firstband", "boltz_calc_also_dos", "boltz_dos_adpt_smr", "boltz_dos_adpt_smr_fac",
    "boltz_dos_adpt_smr_max", "boltz_dos_energy_max", "boltz_dos_energy_min", "boltz_dos_energy_step",
    "boltz_dos_smr_fixed_en_width", "boltz_dos_smr_type", "boltz_kmesh", "boltz_kmesh_spacing", "boltz_mu_max",
    "boltz_mu_min", "boltz_mu_step", "boltz_relax_time", "boltz_tdf_energy_step", "boltz_tdf_smr_fixed_en_width",
    "boltz_tdf_smr_type", "boltz_temp_max", "boltz_temp_min", "boltz_temp_step", "boltzwann", "calc_only_a",
    "conv_noise_amp", "conv_noise_num", "conv_tol", "conv_window", "cp_pp", "degen_thr", "devel_flag",
    "dis_conv_tol", "dis_conv_window", "dis_froz_max", "dis_froz_min", "dis_mix_ratio", "dis_num_iter",
    "dis_spheres_first_wann", "dis_spheres_num", "dis_win_max", "dis_win_min", "dist_cutoff", "dist_cutoff_hc",
    "dist_cutoff_mode", "dos", "dos_adpt_smr", "dos_adpt_smr_fac", "dos_adpt_smr_max", "dos_energy_max",
    "dos_energy_min", "dos_energy_step", "dos_kmesh", "dos_kmesh_spacing", "dos_project", "dos_smr_fixed_en_width",
    "dos_smr_type", "dos_task", "effective_model", "energy_unit", "exclude_bands", "fermi_energy",
    "fermi_energy_max", "fermi_energy_min", "fermi_energy_step", "fermi_surface_num_points", "fermi_surface_plot",
    "fermi_surface_plot_format", "fixed_step", "gamma_only", "geninterp", "geninterp_alsofirstder",
    "geninterp_single_file", "guiding_centres", "gyrotropic", "gyrotropic_band_list", "gyrotropic_box_b1",
    "gyrotropic_box_b2", "gyrotropic_box_b3", "gyrotropic_box_center", "gyrotropic_degen_thresh",
    "gyrotropic_eigval_max", "gyrotropic_freq_max", "gyrotropic_freq_min", "gyrotropic_freq_step",
    "gyrotropic_kmesh", "gyrotropic_kmesh_spacing", "gyrotropic_smr_fixed_en_width", "gyrotropic_smr_max_arg",
    "gyrotropic_smr_type", "gyrotropic_task", "hr_cutoff", "hr_plot", "iprint", "kdotp_bands", "kdotp_kpoint",
    "kdotp_num_bands", "kmesh", "kmesh_spacing", "kmesh_tol", "kpath", "kpath_bands_colour", "kpath_num_points",
    "kpath_task", "kslice", "kslice_2dkmesh", "kslice_b1", "kslice_b2", "kslice_corner",
    "kslice_fermi_lines_colour", "kslice_task", "kubo_adpt_smr", "kubo_adpt_smr_fac", "kubo_adpt_smr_max",
    "kubo_eigval_max", "kubo_freq_max", "kubo_freq_min", "kubo_freq_step", "kubo_smr_fixed_en_width",
    "kubo_smr_type", "length_unit", "mp_grid", "num_bands", "num_cg_steps", "num_dump_cycles",
    "num_elec_per_state", "num_guide_cycles", "num_iter", "num_no_guide_iter", "num_print_cycles", "num_shells",
    "num_valence_bands", "num_wann", "one_dim_axis", "optimisation", "postproc_setup", "precond", "restart",
    "sc_eta", "sc_phase_conv", "sc_use_eta_corr", "sc_w_thr", "scissors_shift", "search_shells",
    "select_projections", "shc_alpha", "shc_bandshift", "shc_bandshift_energyshift", "shc_bandshift_firstband",
    "shc_beta", "shc_freq_scan", "shc_gamma", "shc_method", "shell_list", "site_symmetry", "skip_b1_tests",
    "slwf_constrain", "slwf_lambda", "slwf_num", "smr_fixed_en_width", "smr_max_arg", "smr_type", "spin",
    "spin_axis_azimuth", "spin_axis_polar", "spin_decomp", "spin_kmesh", "spin_kmesh_spacing", "spin_moment",
    "spinors", "spn_formatted", "symmetrize_eps", "timing_level", "tran_easy_fix", "tran_energy_step",
    "tran_group_threshold", "tran_num_bandc", "tran_num_bb", "tran_num_cc", "tran_num_cell_ll",
    "tran_num_cell_rr", "tran_num_cr", "tran_num_lc", "tran_num_ll", "tran_num_rr", "tran_read_ht",
    "tran_use_same_lead", "tran_win_max", "tran_win_min", "tran_write_ht", "transl_inv", "translate_home_cell",
    "translation_centre_frac", "transport", "transport_mode", "trial_step", "uhu_formatted", "unlucky",
    "use_bloch_phases", "use_degen_pert", "use_ws_distance", "wanint_kpoint_file", "wannier_plot",
    "wannier_plot_format", "wannier_plot_list", "wannier_plot_mode", "wannier_plot_radius",
    "wannier_plot_scale", "wannier_plot_spinor_mode", "wannier_plot_spinor_phase", "wannier_plot_supercell",
    "write_bvec", "write_hr", "write_hr_diag", "write_proj", "write_r2mn", "write_rmn", "write_tb",
    "write_u_matrices", "write_vdw_data", "write_xyz", "ws_distance_tol", "ws_search_size", "wvfn_formatted",
};
const char* const kBlocks[] = {"atoms_cart", "atoms_frac", "dis_spheres", "kpoint_path", "kpoints",
                               "nnkpts", "projections", "slwf_centres", "unit_cell_cart"};

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && s[a] == ' ') ++a;
  while (b > a && s[b - 1] == ' ') --b;
  return s.substr(a, b - a);
}

std::vector<std::string> split_ws(const std::string& s, bool commas) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : s) {
    if (c == ' ' || (commas && c == ',')) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur += c;
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

}  // namespace

int read_win(const std::string& path, WinFile& out, std::string& err) {
  std::ifstream f(path);
  if (!f) {
    err = "Error: Problem opening input file " + path;
    return 6;
  }
  static const std::set<std::string> keywords(std::begin(kKeywords), std::end(kKeywords));
  static const std::set<std::string> blocks(std::begin(kBlocks), std::end(kBlocks));
  std::vector<std::string> lines;
  std::string raw;
  while (std::getline(f, raw)) {
    for (auto& c : raw) {
      if (c == '\t' || c == '\r') c = ' ';
      c = (char)std::tolower((unsigned char)c);
    }
    std::string s = trim(raw);
    if (s.empty() || s[0] == '!' || s[0] == '#') continue;
    const size_t cut = s.find_first_of("!#");
    if (cut != std::string::npos) s = trim(s.substr(0, cut));
    if (!s.empty()) lines.push_back(s);
  }
  out = WinFile();
  std::set<std::string> seen;
  for (size_t i = 0; i < lines.size(); ++i) {
    const std::string& s = lines[i];
    std::vector<std::string> w = split_ws(s, false);
    if (w[0] == "begin") {
      if (w.size() < 2) {
        err = "Error: Found begin without a block name in input file";
        return 5;
      }
      const std::string name = w[1];
      std::vector<std::string> body;
      size_t j = i + 1;
      bool closed = false;
      for (; j < lines.size(); ++j) {
        std::vector<std::string> e = split_ws(lines[j], false);
        if (e[0] == "end") {
          if (e.size() < 2 || e[1] != name) {
            err = "Error: Ending tag for " + name + " not found";
            return 5;
          }
          closed = true;
          break;
        }
        body.push_back(lines[j]);
      }
      if (!closed) {
        err = "Error: Ending tag for " + name + " not found";
        return 5;
      }
      if (!blocks.count(name)) {
        err = "Unrecognised keyword(s) in input file, see also output file (block " + name + ")";
        return 5;
      }
      if (out.blocks.count(name)) {
        err = "Error: Found tag begin " + name + " more than once in input file";
        return 5;
      }
      out.blocks[name] = body;
      i = j;
      continue;
    }
    // keyword: letters, digits, '_' up to '=', ':' or a blank
    size_t k = 0;
    while (k < s.size() && (std::isalnum((unsigned char)s[k]) || s[k] == '_')) ++k;
    const std::string key = s.substr(0, k);
    std::string rest = trim(s.substr(k));
    if (key.empty() || (k < s.size() && s[k] != '=' && s[k] != ':' && s[k] != ' ')) {
      err = "Unrecognised keyword(s) in input file, see also output file (" + s + ")";
      return 5;
    }
    if (!rest.empty() && (rest[0] == '=' || rest[0] == ':')) rest = trim(rest.substr(1));
    const bool engine_key = key.compare(0, 4, "gpu_") == 0;
    if (!keywords.count(key) && !engine_key) {
      err = "Unrecognised keyword(s) in input file, see also output file (" + key + ")";
      return 5;
    }
    if (seen.count(key)) {
      err = "Error: Found keyword " + key + " more than once in input file";
      return 5;
    }
    seen.insert(key);
    out.keys.emplace_back(key, rest);
  }
  return 0;
}

bool parse_real(const std::string& text, double& v) {
  std::vector<std::string> w = split_ws(text, true);
  if (w.empty()) return false;
  std::string s = w[0];
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  v = std::strtod(s.c_str(), &end);
  return end && *end == '\0' && end != s.c_str();
}

bool parse_int(const std::string& text, int& v) {
  std::vector<std::string> w = split_ws(text, true);
  if (w.empty()) return false;
  char* end = nullptr;
  const long x = std::strtol(w[0].c_str(), &end, 10);
  if (!end || *end != '\0' || end == w[0].c_str()) return false;
  v = (int)x;
  return true;
}

bool parse_logical(const std::string& text, bool& v) {
  if (text.find('t') != std::string::npos) {
    v = true;
    return true;
  }
  if (text.find('f') != std::string::npos) {
    v = false;
    return true;
  }
  return false;
}

bool parse_reals(const std::string& text, std::vector<double>& v) {
  v.clear();
  for (const std::string& w : split_ws(text, true)) {
    double x;
    if (!parse_real(w, x)) return false;
    v.push_back(x);
  }
  return !v.empty();
}

bool parse_range_vector(const std::string& text, std::vector<int>& v) {
  v.clear();
  for (const std::string& w : split_ws(text, true)) {
    const size_t dash = w.find('-', 1);
    if (dash == std::string::npos) {
      int x;
      if (!parse_int(w, x)) return false;
      v.push_back(x);
    } else {
      int a, b;
      if (!parse_int(w.substr(0, dash), a) || !parse_int(w.substr(dash + 1), b) || b < a) return false;
      for (int x = a; x <= b; ++x) v.push_back(x);
    }
  }
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return !v.empty();
}

namespace {

// one Fortran unformatted sequential record: 4-byte length, payload, 4-byte length
void put_record(std::FILE* f, const void* data, size_t bytes) {
  const int32_t n = (int32_t)bytes;
  std::fwrite(&n, 4, 1, f);
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fwrite(&n, 4, 1, f);
}

template <class T>
void put_scalar(std::FILE* f, T v) {
  put_record(f, &v, sizeof(T));
}

}  // namespace

int write_chk(const std::string& path, const ChkData& d, std::string& err) {
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    err = "Error: Problem opening checkpoint file " + path;
    return 6;
  }
  const int nb = d.num_bands, nk = d.num_kpts, nw = d.num_wann, nn = d.nntot;
  std::string header = d.header;
  header.resize(33, ' ');
  put_record(f, header.data(), 33);
  put_scalar<int32_t>(f, nb);
  put_scalar<int32_t>(f, (int32_t)d.exclude_bands.size());
  std::vector<int32_t> ex(d.exclude_bands.begin(), d.exclude_bands.end());
  put_record(f, ex.data(), ex.size() * 4);
  // ((real_lattice(i, j), i = 1, 3), j = 1, 3) with real_lattice(i, :) = a_i
  double lat[9], rec[9], rl[9], vol = 0.0;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) lat[j * 3 + i] = d.real_lattice[i * 3 + j];
  put_record(f, lat, sizeof lat);
  recip_lattice(d.real_lattice, rl, &vol);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) rec[j * 3 + i] = rl[i * 3 + j];
  put_record(f, rec, sizeof rec);
  put_scalar<int32_t>(f, nk);
  const int32_t mp[3] = {d.mp_grid[0], d.mp_grid[1], d.mp_grid[2]};
  put_record(f, mp, sizeof mp);
  put_record(f, d.kpt_latt, (size_t)nk * 3 * sizeof(double));
  put_scalar<int32_t>(f, nn);
  put_scalar<int32_t>(f, nw);
  std::string cp = d.checkpoint;
  cp.resize(20, ' ');
  put_record(f, cp.data(), 20);
  put_scalar<int32_t>(f, d.have_disentangled ? 1 : 0);
  if (d.have_disentangled) {
    put_scalar<double>(f, d.omega_invariant);
    std::vector<int32_t> lw(d.lwindow.begin(), d.lwindow.end());
    put_record(f, lw.data(), lw.size() * 4);
    std::vector<int32_t> nd(d.ndimwin.begin(), d.ndimwin.end());
    put_record(f, nd.data(), nd.size() * 4);
    put_record(f, d.u_opt, (size_t)nb * nw * nk * 16);
  }
  put_record(f, d.u, (size_t)nw * nw * nk * 16);
  // ((((m(i, j, b, k), i = 1, nw), j = 1, nw), b = 1, nntot), k = 1, nk) of the leading block
  std::vector<double> m((size_t)nw * nw * nn * nk * 2);
  for (size_t kb = 0; kb < (size_t)nn * nk; ++kb)
    for (int j = 0; j < nw; ++j)
      for (int i = 0; i < nw; ++i) {
        const double* src = d.m + 2 * ((kb * d.ldm + j) * d.ldm + i);
        double* dst = &m[2 * ((kb * nw + j) * nw + i)];
        dst[0] = src[0];
        dst[1] = src[1];
      }
  put_record(f, m.data(), m.size() * sizeof(double));
  put_record(f, d.centres, (size_t)3 * nw * sizeof(double));
  put_record(f, d.spreads, (size_t)nw * sizeof(double));
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  if (!ok) {
    err = "Error: Problem writing checkpoint file " + path;
    return 6;
  }
  return 0;
}

}  // namespace w90g
