// A C++ caller of the library mode, written against include/wannier90_gb300.h the way a
// DFT code uses Wannier90's C++ prototypes (src/wannier90.hh): the system through
// cset_option, cinput_setopt, the remaining keywords from <seed>.win through
// cinput_reader, the neighbour list through cget_nn / cget_nnkp; then the caller's own
// arrays (eigenvalues, overlaps gathered per neighbour, projections) through cset_*,
// cdisentangle, cwannierise, cget_centres / cget_spreads.  Test program of
// tests/test_libv2.py; it reads the seed files itself, as such a caller holds the data in
// memory.
//
//   gaas_driver <seed> <nb> <nw> <n1> <n2> <n3> a11 a12 a13 a21 a22 a23 a31 a32 a33
// prints one line per WF: x y z spread, then "ierr <disentangle> <wannierise>".
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "wannier90_gb300.h"

using cplx = std::complex<double>;

static void die(const std::string& msg) {
  std::cerr << msg << std::endl;
  std::exit(2);
}

int main(int argc, char** argv) {
  if (argc != 16) die("usage: gaas_driver seed nb nw n1 n2 n3 a11 .. a33");
  const std::string seed = argv[1];
  const int nb = std::atoi(argv[2]), nw = std::atoi(argv[3]);
  int mp[3] = {std::atoi(argv[4]), std::atoi(argv[5]), std::atoi(argv[6])};
  double cell[3][3];
  for (int i = 0; i < 9; ++i) cell[i / 3][i % 3] = std::atof(argv[7 + i]);
  const int nk = mp[0] * mp[1] * mp[2];
  // k-points of the Monkhorst-Pack mesh, last index fastest
  std::vector<double> kpt;
  for (int a = 0; a < mp[0]; ++a)
    for (int b = 0; b < mp[1]; ++b)
      for (int c = 0; c < mp[2]; ++c) {
        kpt.push_back(double(a) / mp[0]);
        kpt.push_back(double(b) / mp[1]);
        kpt.push_back(double(c) / mp[2]);
      }

  // ---- setup
  void* w90 = w90_create();
  cset_option(w90, "kpoints", kpt.data(), nk, 3);
  cset_option(w90, "mp_grid", mp);
  cset_option(w90, "num_bands", nb);
  cset_option(w90, "num_kpts", nk);
  cset_option(w90, "num_wann", nw);
  cset_option(w90, "unit_cell_cart", &cell[0][0], 3, 3);
  int ierr = 0;
  cinput_setopt(w90, seed, ierr);
  if (ierr) die("cinput_setopt: " + std::string(w90g_last_error(w90)));
  cinput_reader(w90, ierr);
  if (ierr) die("cinput_reader: " + std::string(w90g_last_error(w90)));
  int nn = 0;
  cget_nn(w90, nn);
  std::vector<int> nnkp((size_t)nn * nk);
  cget_nnkp(w90, nnkp.data());

  // ---- the caller's data: eigenvalues [k][band], projections [k][w][band], overlaps for
  // every (k, k2) pair the file holds, gathered per neighbour [k][nn][n][m]
  std::vector<double> eig((size_t)nk * nb);
  {
    std::ifstream f(seed + ".eig");
    for (int k = 0; k < nk; ++k)
      for (int n = 0; n < nb; ++n) {
        int i, j;
        double e;
        if (!(f >> i >> j >> e) || i != n + 1 || j != k + 1) die("bad .eig");
        eig[(size_t)k * nb + n] = e;
      }
  }
  std::vector<cplx> amat((size_t)nk * nw * nb);
  {
    std::ifstream f(seed + ".amn");
    std::string line;
    std::getline(f, line);
    int b0, k0, w0;
    f >> b0 >> k0 >> w0;
    if (b0 != nb || k0 != nk || w0 != nw) die("bad .amn header");
    for (size_t r = 0; r < amat.size(); ++r) {
      int m, n, k;
      double re, im;
      if (!(f >> m >> n >> k >> re >> im)) die("bad .amn");
      amat[((size_t)(k - 1) * nw + (n - 1)) * nb + (m - 1)] = cplx(re, im);
    }
  }
  std::vector<cplx> mloc((size_t)nk * nn * nb * nb);
  {
    std::ifstream f(seed + ".mmn");
    std::string line;
    std::getline(f, line);
    int b0, k0, n0;
    f >> b0 >> k0 >> n0;
    if (b0 != nb || k0 != nk || n0 != nn) die("bad .mmn header");
    std::vector<cplx> blk((size_t)nb * nb);
    for (int r = 0; r < nk * nn; ++r) {
      int k1, k2, g1, g2, g3;
      if (!(f >> k1 >> k2 >> g1 >> g2 >> g3)) die("bad .mmn block header");
      for (size_t e = 0; e < blk.size(); ++e) {
        double re, im;
        if (!(f >> re >> im)) die("bad .mmn values");
        blk[e] = cplx(re, im);
      }
      // the neighbour slot of k1 whose k+b is k2 (one per k2 on this mesh)
      int slot = -1;
      for (int b = 0; b < nn; ++b)
        if (nnkp[(size_t)b * nk + (k1 - 1)] == k2) slot = b;
      if (slot < 0) die("k2 is not a neighbour");
      std::copy(blk.begin(), blk.end(), mloc.begin() + ((size_t)(k1 - 1) * nn + slot) * nb * nb);
    }
  }

  // ---- run
  std::vector<cplx> umat((size_t)nk * nw * nw);
  std::vector<double> centres((size_t)nw * 3), spreads(nw);
  cset_eigval(w90, eig.data());
  cset_m_local(w90, mloc.data());
  cset_u_opt(w90, amat.data());
  cset_u_matrix(w90, umat.data());
  int ierr_dis = 0, ierr_wann = 0;
  cdisentangle(w90, ierr_dis);
  if (ierr_dis > 0) die("cdisentangle: " + std::string(w90g_last_error(w90)));
  cwannierise(w90, ierr_wann);
  if (ierr_wann > 0) die("cwannierise: " + std::string(w90g_last_error(w90)));
  cget_centres(w90, centres.data());
  cget_spreads(w90, spreads.data());
  w90_delete(w90);
  std::printf("\n");
  for (int n = 0; n < nw; ++n)
    std::printf("%.12f %.12f %.12f %.12f\n", centres[3 * n], centres[3 * n + 1], centres[3 * n + 2], spreads[n]);
  std::printf("ierr %d %d\n", ierr_dis, ierr_wann);
  return 0;
}
