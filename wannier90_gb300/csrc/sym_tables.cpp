#include "sym_tables.h"

namespace w90g {

int build_sym_tables(int nw, int nb, int nsym, int nkirr, int nk, const int* ik2ir, const int* ir2ik,
                     const int* kptsym, const double* d_wann, const double* d_band, SymTables& t, std::string& msg) {
  if (nsym < 1 || nkirr < 1 || nkirr > nk || nw < 1 || nb < nw || !ik2ir || !ir2ik || !kptsym || !d_wann || !d_band) {
    msg = "Error: symmetry data missing or inconsistent (sitesym_read)";
    return 6;
  }
  for (int k = 0; k < nk; ++k)
    if (ik2ir[k] < 1 || ik2ir[k] > nkirr) {
      msg = "Error: ik2ir out of range (sitesym_read)";
      return 6;
    }
  for (int ir = 0; ir < nkirr; ++ir) {
    if (ir2ik[ir] < 1 || ir2ik[ir] > nk) {
      msg = "Error: ir2ik out of range (sitesym_read)";
      return 6;
    }
    if (ik2ir[ir2ik[ir] - 1] != ir + 1) {
      msg = "Error: ik2ir and ir2ik disagree (sitesym_read)";
      return 6;
    }
  }
  for (long i = 0; i < (long)nsym * nkirr; ++i)
    if (kptsym[i] < 1 || kptsym[i] > nk) {
      msg = "Error: kptsym out of range (sitesym_read)";
      return 6;
    }
  const size_t WW = (size_t)nw * nw, BB = (size_t)nb * nb;
  std::vector<int> slot((size_t)nsym * nkirr, -1);
  SymTables r;
  auto slot_of = [&](int ir, int isym) {
    int& sl = slot[(size_t)ir * nsym + isym];
    if (sl < 0) {
      sl = (int)(r.d.size() / (2 * WW));
      const double* a = d_wann + 2 * WW * ((size_t)ir * nsym + isym);
      const double* b = d_band + 2 * BB * ((size_t)ir * nsym + isym);
      r.d.insert(r.d.end(), a, a + 2 * WW);
      r.db.insert(r.db.end(), b, b + 2 * BB);
    }
    return sl;
  };
  r.nir = nkirr;
  r.nsym = nsym;
  r.ik.resize(nkirr);
  std::vector<char> done(nk, 0);
  // star members in first-occurrence order (sitesym_symmetrize_rotation / _gradient
  // mode 1 / _u_matrix, :119-190, :222-240, :305-322)
  for (int ir = 0; ir < nkirr; ++ir) {
    r.ik[ir] = ir2ik[ir] - 1;
    done[r.ik[ir]] = 1;
    r.moff.push_back((int)r.mem.size() / 2);
    for (int isym = 1; isym < nsym; ++isym) {
      const int irk = kptsym[(size_t)ir * nsym + isym] - 1;
      if (done[irk]) continue;
      done[irk] = 1;
      r.mem.push_back(irk);
      r.mem.push_back(slot_of(ir, isym));
    }
  }
  r.moff.push_back((int)r.mem.size() / 2);
  std::vector<char> member(nk, 0);
  for (size_t m = 0; m < r.mem.size(); m += 2) member[r.mem[m]] = 1;
  for (int k = 0; k < nk; ++k) {
    if (!done[k]) {
      msg = "error in sitesym_symmetrize_rotation";
      return 1;
    }
    // the members are exactly the k whose irreducible point is another k (mode 1 zeroes those)
    const bool irr = ir2ik[ik2ir[k] - 1] - 1 == k;
    if (irr == (member[k] != 0)) {
      msg = "Error: k-point stars and ik2ir disagree (sitesym_read)";
      return 6;
    }
  }
  // little groups {R : R k = k} in isym order, the first symmetry included (symmetrize_ukirr, :451-470)
  for (int ir = 0; ir < nkirr; ++ir) {
    r.goff.push_back((int)r.grp.size() / 2);
    for (int isym = 0; isym < nsym; ++isym)
      if (kptsym[(size_t)ir * nsym + isym] - 1 == r.ik[ir]) {
        r.grp.push_back(isym);
        r.grp.push_back(slot_of(ir, isym));
      }
  }
  r.goff.push_back((int)r.grp.size() / 2);
  t = std::move(r);
  return 0;
}

}  // namespace w90g
