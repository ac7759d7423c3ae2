// Host-side b-vector tables: restatement of kmesh_get (src/kmesh.F90:61-740) for the
// automatic shell choice, including the cell search order of kmesh_supercell_sort
// (:984-1038, ties broken as internal_maxloc :1866-1883), the shell-parallelism test and
// B1 weights of kmesh_shell_automatic (:1107-1432), and the neighbour lists (:362-390).
#include "kmesh.h"

#include <algorithm>
#include <cmath>
#include <cstdio>

namespace w90g {

static const int kNsupcell = 5;  // src/kmesh.F90:55

void recip_lattice(const double a[9], double b[9], double* volume) {
  // rows b_i = 2 pi (a_j x a_k) / det  (utility_recip_lattice_base, src/utility.F90:313-336)
  auto cross = [](const double* u, const double* v, double* w) {
    w[0] = u[1] * v[2] - u[2] * v[1];
    w[1] = u[2] * v[0] - u[0] * v[2];
    w[2] = u[0] * v[1] - u[1] * v[0];
  };
  double c[9];
  cross(a + 3, a + 6, c);
  cross(a + 6, a + 0, c + 3);
  cross(a + 0, a + 3, c + 6);
  const double det = a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
  const double twopi = 2.0 * M_PI;
  for (int i = 0; i < 9; ++i) b[i] = twopi * c[i] / det;
  if (volume) *volume = std::fabs(det);
}

// symmetric eigen-decomposition (cyclic Jacobi) of a small n x n matrix, row-major
static void sym_eig(int n, std::vector<double>& A, std::vector<double>& V) {
  V.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double th = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(1.0 + th * th));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
}

int kmesh_get(const double real_lattice[9], const double* kpt_latt, int K, int search_shells,
              double tol, KmeshInfo& out, std::string& err) {
  double recip[9];
  double vol = 0;
  recip_lattice(real_lattice, recip, &vol);
  if (vol < 1e-5) {
    err = "Found almost zero Volume in utility_recip_lattice";
    return 1;
  }
  auto to_cart = [&](const double* f, double* c) {
    for (int i = 0; i < 3; ++i) c[i] = f[0] * recip[i] + f[1] * recip[3 + i] + f[2] * recip[6 + i];
  };
  // kmesh_supercell_sort
  const int n = kNsupcell;
  std::vector<std::array<int, 3>> lmn;
  lmn.push_back({0, 0, 0});
  for (int l = -n; l <= n; ++l)
    for (int m = -n; m <= n; ++m)
      for (int k = -n; k <= n; ++k) {
        if (l == 0 && m == 0 && k == 0) continue;
        lmn.push_back({l, m, k});
      }
  const int N = (int)lmn.size();
  std::vector<double> dist(N);
  std::vector<std::array<double, 3>> cellc(N);
  for (int i = 0; i < N; ++i) {
    double f[3] = {(double)lmn[i][0], (double)lmn[i][1], (double)lmn[i][2]};
    double c[3];
    to_cart(f, c);
    cellc[i] = {c[0], c[1], c[2]};
    dist[i] = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  }
  std::vector<int> order(N);
  {
    std::vector<double> d = dist;
    std::vector<char> alive(N, 1);
    for (int pos = N - 1; pos >= 0; --pos) {
      int g = -1;
      double mx = -2.0;
      for (int i = 0; i < N; ++i)
        if (alive[i] && d[i] > mx) {
          mx = d[i];
          g = i;
        }
      int idx = g;
      for (int i = 0; i < N; ++i)
        if (alive[i] && std::fabs(d[i] - d[g]) < 1e-8 && i < idx) idx = i;
      order[pos] = idx;
      alive[idx] = 0;
      d[idx] = -1.0;
    }
  }
  std::vector<std::array<double, 3>> lmn_c(N);
  std::vector<std::array<int, 3>> lmn_s(N);
  for (int i = 0; i < N; ++i) {
    lmn_c[i] = cellc[order[i]];
    lmn_s[i] = lmn[order[i]];
  }
  std::vector<std::array<double, 3>> kc(K);
  for (int k = 0; k < K; ++k) {
    double c[3];
    to_cart(kpt_latt + 3 * k, c);
    kc[k] = {c[0], c[1], c[2]};
  }
  // shell distances (src/kmesh.F90:129-158)
  const double eta = 99999999.0;
  std::vector<double> dnn(search_shells);
  std::vector<int> multi(search_shells);
  double dnn0 = 0.0, dnn1 = eta;
  for (int s = 0; s < search_shells; ++s) {
    int counter = 0;
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < N; ++i) {
        const double x = kc[k][0] + lmn_c[i][0], y = kc[k][1] + lmn_c[i][1], z = kc[k][2] + lmn_c[i][2];
        const double dd = std::sqrt(x * x + y * y + z * z);
        if (dd > tol && dd > dnn0 + tol) {
          if (dd < dnn1 - tol) {
            dnn1 = dd;
            counter = 0;
          }
          if (dd > dnn1 - tol && dd < dnn1 + tol) ++counter;
        }
      }
    dnn[s] = dnn1;
    multi[s] = counter;
    dnn0 = dnn1;
    dnn1 = eta;
  }
  // b-vectors of a shell around k-point 1 (kmesh_get_bvectors, :1041-1104)
  auto get_bvectors = [&](int s, std::vector<std::array<double, 3>>& bv) {
    bv.clear();
    for (int i = 0; i < N; ++i) {
      for (int k2 = 0; k2 < K; ++k2) {
        const double v[3] = {lmn_c[i][0] + kc[k2][0], lmn_c[i][1] + kc[k2][1], lmn_c[i][2] + kc[k2][2]};
        const double dx = kc[0][0] - v[0], dy = kc[0][1] - v[1], dz = kc[0][2] - v[2];
        const double dd = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (dd >= dnn[s] * (1.0 - tol) && dd <= dnn[s] * (1.0 + tol))
          bv.push_back({v[0] - kc[0][0], v[1] - kc[0][1], v[2] - kc[0][2]});
        if ((int)bv.size() == multi[s]) return;
      }
    }
  };
  // kmesh_shell_automatic
  const double target[6] = {1, 1, 1, 0, 0, 0};
  std::vector<int> shell_list;
  std::vector<std::vector<std::array<double, 3>>> shell_b;
  std::vector<double> bweight;
  bool b1sat = false;
  for (int s = 0; s < search_shells && !b1sat; ++s) {
    std::vector<std::array<double, 3>> bv;
    get_bvectors(s, bv);
    bool lpar = false;
    for (auto& b1 : bv)
      for (auto& prev : shell_b)
        for (auto& b2 : prev) {
          const double d12 = b1[0] * b2[0] + b1[1] * b2[1] + b1[2] * b2[2];
          const double n1 = b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2];
          const double n2 = b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2];
          if (std::fabs(std::fabs(d12 / std::sqrt(n1 * n2)) - 1.0) < 1e-6) lpar = true;
        }
    if (lpar) continue;
    shell_list.push_back(s);
    shell_b.push_back(bv);
    const int ns = (int)shell_list.size();
    std::vector<double> amat(6 * ns, 0.0);  // row-major 6 x ns
    for (int j = 0; j < ns; ++j)
      for (auto& b : shell_b[j]) {
        amat[0 * ns + j] += b[0] * b[0];
        amat[1 * ns + j] += b[1] * b[1];
        amat[2 * ns + j] += b[2] * b[2];
        amat[3 * ns + j] += b[0] * b[1];
        amat[4 * ns + j] += b[1] * b[2];
        amat[5 * ns + j] += b[2] * b[0];
      }
    // singular values of amat via eig(A^T A); least-squares weights via its pseudo-inverse
    std::vector<double> ata(ns * ns, 0.0), V;
    for (int i = 0; i < ns; ++i)
      for (int j = 0; j < ns; ++j)
        for (int r = 0; r < 6; ++r) ata[i * ns + j] += amat[r * ns + i] * amat[r * ns + j];
    sym_eig(ns, ata, V);
    bool small = false;
    for (int i = 0; i < ns; ++i)
      if (std::sqrt(std::max(ata[i * ns + i], 0.0)) < 1e-5) small = true;
    if (small) {
      if (ns == 1) {
        err = "kmesh_shell_automatic: Singular Value Decomposition has found a very small singular value";
        return 1;
      }
      shell_list.pop_back();
      shell_b.pop_back();
      continue;
    }
    std::vector<double> atb(ns, 0.0), w(ns, 0.0);
    for (int i = 0; i < ns; ++i)
      for (int r = 0; r < 6; ++r) atb[i] += amat[r * ns + i] * target[r];
    for (int i = 0; i < ns; ++i) {
      double acc = 0.0;
      for (int l = 0; l < ns; ++l) {
        double vt_atb = 0.0;
        for (int j = 0; j < ns; ++j) vt_atb += V[j * ns + l] * atb[j];
        acc += V[i * ns + l] * vt_atb / ata[l * ns + l];
      }
      w[i] = acc;
    }
    b1sat = true;
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        double delta = 0.0;
        for (int sh = 0; sh < ns; ++sh)
          for (auto& b : shell_b[sh]) delta += w[sh] * b[i] * b[j];
        if (i == j && std::fabs(delta - 1.0) > tol) b1sat = false;
        if (i != j && std::fabs(delta) > tol) b1sat = false;
      }
    if (b1sat) bweight = w;
  }
  if (!b1sat) {
    err = "Unable to satisfy B1 with any of the searched shells";
    return 1;
  }
  int nntot = 0;
  for (int s : shell_list) nntot += multi[s];
  if (nntot > 12) {  // num_nnmax (src/types.F90:116)
    err = "kmesh_get: something wrong, found too many nearest neighbours";
    return 1;
  }
  out.nntot = nntot;
  out.K = K;
  out.wb.clear();
  for (size_t i = 0; i < shell_list.size(); ++i)
    for (int j = 0; j < multi[shell_list[i]]; ++j) out.wb.push_back(bweight[i]);
  out.nnlist.assign((size_t)K * nntot, -1);
  out.nncell.assign((size_t)K * nntot * 3, 0);
  out.bk.assign((size_t)K * nntot * 3, 0.0);
  for (int k = 0; k < K; ++k) {
    int nnx = 0;
    for (int s : shell_list) {
      int cnt = 0;
      bool done = false;
      for (int i = 0; i < N && !done; ++i) {
        for (int k2 = 0; k2 < K; ++k2) {
          const double v[3] = {lmn_c[i][0] + kc[k2][0], lmn_c[i][1] + kc[k2][1], lmn_c[i][2] + kc[k2][2]};
          const double dx = kc[k][0] - v[0], dy = kc[k][1] - v[1], dz = kc[k][2] - v[2];
          const double dd = std::sqrt(dx * dx + dy * dy + dz * dz);
          if (dd >= dnn[s] * (1 - tol) && dd <= dnn[s] * (1 + tol)) {
            if (nnx >= nntot) {
              err = "kmesh_get: too many neighbours for a k-point";
              return 1;
            }
            out.nnlist[(size_t)k * nntot + nnx] = k2;
            for (int c = 0; c < 3; ++c) {
              out.nncell[((size_t)k * nntot + nnx) * 3 + c] = lmn_s[i][c];
              out.bk[((size_t)k * nntot + nnx) * 3 + c] = v[c] - kc[k][c];
            }
            ++nnx;
            ++cnt;
          }
          if (cnt == multi[s]) {
            done = true;
            break;
          }
        }
      }
    }
    if (nnx != nntot) {
      err = "kmesh_get: wrong number of neighbours for a k-point";
      return 1;
    }
  }
  // B1 completeness for every k-point (:450-490)
  for (int k = 0; k < K; ++k)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double dd = 0.0;
        for (int b = 0; b < nntot; ++b)
          dd += out.wb[b] * out.bk[((size_t)k * nntot + b) * 3 + i] * out.bk[((size_t)k * nntot + b) * 3 + j];
        if ((i == j && std::fabs(dd - 1.0) > tol) || (i != j && std::fabs(dd) > tol)) {
          err = "Eq. (B1) not satisfied in kmesh_get";
          return 1;
        }
      }
  out.wbtot = 0.0;
  for (double w : out.wb) out.wbtot += w;
  // b directions without inversion partners, from the first k-point (:505-528), and
  // their index in every k-point's neighbour list (:561-577, last match wins)
  auto compar = [](const double* a, const double* b, int& pos, int& neg) {
    double rp = 0.0, rm = 0.0;
    for (int i = 0; i < 3; ++i) {
      rp += (a[i] - b[i]) * (a[i] - b[i]);
      rm += (a[i] + b[i]) * (a[i] + b[i]);
    }
    pos = std::fabs(rp) < 1e-8;
    neg = std::fabs(rm) < 1e-8;
  };
  out.nnh = nntot / 2;
  out.bka.clear();
  for (int nn = 0; nn < nntot; ++nn) {
    const double* b = &out.bk[(size_t)nn * 3];
    bool found = false;
    for (size_t na = 0; na < out.bka.size() / 3; ++na) {
      int pos, neg;
      compar(&out.bka[na * 3], b, pos, neg);
      if (neg) found = true;
    }
    if (!found) out.bka.insert(out.bka.end(), b, b + 3);
  }
  if ((int)out.bka.size() != 3 * out.nnh) {
    err = "Did not find right number of bk directions";
    return 1;
  }
  out.neigh.assign((size_t)K * out.nnh, -1);
  for (int k = 0; k < K; ++k)
    for (int na = 0; na < out.nnh; ++na) {
      for (int nn = 0; nn < nntot; ++nn) {
        int pos, neg;
        compar(&out.bka[(size_t)na * 3], &out.bk[((size_t)k * nntot + nn) * 3], pos, neg);
        if (pos) out.neigh[(size_t)k * out.nnh + na] = nn;
      }
      if (out.neigh[(size_t)k * out.nnh + na] < 0) {
        err = "kmesh_get: failed to find neighbours for this kpoint";
        return 1;
      }
    }
  return 0;
}

int ws_vectors(const double real_lattice[9], const int mp_grid[3], const int search_size[3],
               double dist_tol, std::vector<int>& irvec, std::vector<int>& ndegen, std::string& err) {
  // metric g_ij = a_i . a_j (utility_metric, src/utility.F90:397-423)
  double g[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double a = 0.0;
      for (int l = 0; l < 3; ++l) a += real_lattice[i * 3 + l] * real_lattice[j * 3 + l];
      g[i * 3 + j] = a;
    }
  const int s1 = search_size[0], s2 = search_size[1], s3 = search_size[2];
  const int ndist = (2 * (s1 + 1) + 1) * (2 * (s2 + 1) + 1) * (2 * (s3 + 1) + 1);
  const int centre = (ndist - 1) / 2;   // i1 = i2 = i3 = 0
  const double tol2 = dist_tol * dist_tol;
  std::vector<double> dist(ndist);
  irvec.clear();
  ndegen.clear();
  for (int n1 = -s1 * mp_grid[0]; n1 <= s1 * mp_grid[0]; ++n1)
    for (int n2 = -s2 * mp_grid[1]; n2 <= s2 * mp_grid[1]; ++n2)
      for (int n3 = -s3 * mp_grid[2]; n3 <= s3 * mp_grid[2]; ++n3) {
        int c = 0;
        double dmin = 1e300;
        for (int i1 = -s1 - 1; i1 <= s1 + 1; ++i1)
          for (int i2 = -s2 - 1; i2 <= s2 + 1; ++i2)
            for (int i3 = -s3 - 1; i3 <= s3 + 1; ++i3) {
              const double d[3] = {(double)(n1 - i1 * mp_grid[0]), (double)(n2 - i2 * mp_grid[1]),
                                   (double)(n3 - i3 * mp_grid[2])};
              double x = 0.0;
              for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) x += d[i] * g[i * 3 + j] * d[j];
              dist[c++] = x;
              dmin = std::min(dmin, x);
            }
        if (std::fabs(dist[centre] - dmin) < tol2) {
          int deg = 0;
          for (int i = 0; i < ndist; ++i) deg += (std::fabs(dist[i] - dmin) < tol2) ? 1 : 0;
          irvec.push_back(n1);
          irvec.push_back(n2);
          irvec.push_back(n3);
          ndegen.push_back(deg);
        }
      }
  double tot = 0.0;
  for (int d : ndegen) tot += 1.0 / (double)d;
  if (std::fabs(tot - (double)mp_grid[0] * mp_grid[1] * mp_grid[2]) > 1e-8) {
    err = "hamiltonian_wigner_seitz: error in finding Wigner-Seitz points";
    return 1;
  }
  return 0;
}

}  // namespace w90g
