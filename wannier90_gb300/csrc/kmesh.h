// Host-side k-mesh tables (kmesh_info_type, src/types.F90:161-176).
#pragma once
#include <array>
#include <string>
#include <vector>

namespace w90g {

struct KmeshInfo {
  int nntot = 0;
  int K = 0;
  std::vector<int> nnlist;     // [k][b], 0-based index of k+b
  std::vector<int> nncell;     // [k][b][3], G-vector (cell) of k+b
  std::vector<double> wb;      // [b]
  std::vector<double> bk;      // [k][b][3], Cartesian 1/Angstrom
  double wbtot = 0.0;
  int nnh = 0;                 // b directions without inversion partners
  std::vector<double> bka;     // [nnh][3]
  std::vector<int> neigh;      // [k][nnh], index into the k-point's nnlist (0-based)
};

void recip_lattice(const double a[9], double b[9], double* volume);

// real_lattice: rows a_1, a_2, a_3 (Angstrom, row-major); kpt_latt: K x 3 fractional.
int kmesh_get(const double real_lattice[9], const double* kpt_latt, int K, int search_shells,
              double tol, KmeshInfo& out, std::string& err);

// Wigner-Seitz points of the Born-von Karman supercell (hamiltonian_wigner_seitz,
// src/hamiltonian.F90:689-853): irvec [nrpts][3] in the reference's loop order and the
// degeneracies ndegen [nrpts].  Fails when the sum rule sum 1/ndegen = prod mp_grid breaks.
int ws_vectors(const double real_lattice[9], const int mp_grid[3], const int search_size[3],
               double dist_tol, std::vector<int>& irvec, std::vector<int>& ndegen, std::string& err);

}  // namespace w90g
