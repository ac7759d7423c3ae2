// Wannier90 input and checkpoint files on the host: the .win keyword reader behind
// cinput_reader / cinput_reader_special and the .chk writer behind cchkpt.
#pragma once
#include <map>
#include <string>
#include <vector>

namespace w90g {

// A .win file as the reference's tokenizer sees it (w90_readwrite_in_file,
// src/readwrite.F90:2151-2231): lower case, tabs as blanks, '!' / '#' comments and blank
// lines dropped; keyword lines split into keyword and value text
// (w90_readwrite_get_keyword, :2234-2330); begin/end blocks collected by name.
struct WinFile {
  std::vector<std::pair<std::string, std::string>> keys;   // in file order
  std::map<std::string, std::vector<std::string>> blocks;  // block name -> body lines
};

// Reads and tokenizes `path`.  Returns 0, or 6 (file) / 5 (input) with the reference's
// message in err: a missing file, a keyword given twice, an unterminated block, or a
// keyword that neither wannier90.x nor postw90.x accepts
// (w90_readwrite_clean_infile, :1179-1213; the accepted set of :903-1176) unless it
// is one of the engine's own keys (prefix gpu_).
int read_win(const std::string& path, WinFile& out, std::string& err);

// Value parsers for keyword text: a Fortran real ('d' exponents allowed), an integer, a
// logical (the reference's test: a 't' makes it true, else an 'f' false), a list of
// numbers, and a range vector ("1-5, 7 9-10" -> sorted 1-based integers,
// w90_readwrite_get_range_vector).  Return false on malformed text.
bool parse_real(const std::string& text, double& v);
bool parse_int(const std::string& text, int& v);
bool parse_logical(const std::string& text, bool& v);
bool parse_reals(const std::string& text, std::vector<double>& v);
bool parse_range_vector(const std::string& text, std::vector<int>& v);

// Bohr radius in Angstrom for unit_cell_cart given in bohr (src/constants.F90).
constexpr double kBohrAngstrom = 0.52917720859;

// Everything the .chk layout of w90_wannier90_readwrite_write_chkpt
// (src/wannier90_readwrite.F90:2278-2373) records, Fortran-ordered arrays.
struct ChkData {
  std::string header;             // 33 characters ("written on ...")
  int num_bands = 0, num_kpts = 0, nntot = 0, num_wann = 0;
  std::vector<int> exclude_bands;
  double real_lattice[9] = {0};   // rows a_i (Angstrom)
  int mp_grid[3] = {0, 0, 0};
  const double* kpt_latt = nullptr;   // [nk][3]
  std::string checkpoint;         // 'postdis' / 'postwann' (20 characters)
  bool have_disentangled = false;
  double omega_invariant = 0.0;
  std::vector<int> lwindow;       // (nb, nk) 0/1
  std::vector<int> ndimwin;       // (nk)
  const double* u_opt = nullptr;  // complex (nb, nw, nk)
  const double* u = nullptr;      // complex (nw, nw, nk)
  const double* m = nullptr;      // complex (ldm, ldm, nntot, nk): the top-left nw x nw is written
  int ldm = 0;
  const double* centres = nullptr;   // (3, nw)
  const double* spreads = nullptr;   // (nw)
};

// Writes the unformatted sequential .chk (4-byte record markers, little-endian).
int write_chk(const std::string& path, const ChkData& d, std::string& err);

}  // namespace w90g
