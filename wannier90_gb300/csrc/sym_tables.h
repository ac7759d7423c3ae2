// Star and little-group tables of the symmetry-adapted mode, built from sitesym_read's
// data (src/sitesym.F90:698-765) in the reference's loop order.  Host code shared by the
// C ABI (w90g_set_sitesym) and the kernels' tests.
#pragma once
#include <string>
#include <vector>

namespace w90g {

struct SymTables {
  int nir = 0, nsym = 0;
  std::vector<int> ik;              // [nir] irreducible k (0-based)
  std::vector<int> moff, mem;       // star members: mem[2m] = k, mem[2m+1] = slot
  std::vector<int> goff, grp;       // little groups: grp[2g] = isym (0-based), grp[2g+1] = slot
  std::vector<double> d, db;        // slot matrices D(R,k_ir) (nw x nw) and d(R,k_ir) (nb x nb),
                                    // column-major, re/im interleaved
};

// ik2ir[nk], ir2ik[nkirr], kptsym(nsym, nkirr): 1-based, Fortran order; d_wann
// (nw, nw, nsym, nkirr), d_band (nb, nb, nsym, nkirr): Fortran order, (re, im) pairs.
// Returns 0, or the reference's error code with msg: 6 for indices out of range or
// inconsistent, 1 when the stars do not cover the mesh.
int build_sym_tables(int nw, int nb, int nsym, int nkirr, int nk, const int* ik2ir, const int* ir2ik,
                     const int* kptsym, const double* d_wann, const double* d_band, SymTables& t, std::string& msg);

}  // namespace w90g
