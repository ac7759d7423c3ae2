// Readers of the formatted seed files that feed the path: .mmn and .amn (overlap_read,
// src/overlap.F90:234-366) and .eig (w90_readwrite_read_eigvals, src/readwrite.F90:583-635).
//
// The reference reads them record by record with list-directed READs.  At the sizes the
// GPU engine solves (1000 k-points x 8 neighbours x 32^2 bands: 8.2 M overlap records,
// ~300 MB of text) that serial parse takes longer than the solve, so here the file is read
// in one go, its records are indexed with memchr, and the records are converted in
// parallel with std::from_chars (correctly rounded, locale-free; 'd'/'D' exponents of
// Fortran output are accepted).  Each READ of the reference consumes one record and
// ignores trailing items; blank records are skipped, as list-directed input does.
// Placement follows overlap_read: a .mmn block (k, k2, G) goes to the neighbour slot nn
// with nnlist(k,nn) = k2 and nncell(:,k,nn) = G; when two blocks map to one slot the later
// one in the file wins, as in a sequential read.
#include <algorithm>
#include <atomic>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "seedio.h"

namespace w90g {

namespace {

bool load_file(const char* path, std::string& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (n < 0) {
    std::fclose(f);
    return false;
  }
  buf.resize((size_t)n);
  const size_t got = n ? std::fread(&buf[0], 1, (size_t)n, f) : 0;
  std::fclose(f);
  return got == (size_t)n;
}

bool blank(const char* b, const char* e) {
  for (; b < e; ++b)
    if (!(*b == ' ' || *b == '\t' || *b == '\r' || *b == ',')) return false;
  return true;
}

// start/end of every non-blank record (the first `keep_first` records are kept even when
// blank: the title line of .mmn/.amn may be empty)
void index_records(const std::string& buf, int keep_first, std::vector<const char*>& rb,
                   std::vector<const char*>& re) {
  const char* p = buf.data();
  const char* end = p + buf.size();
  int n = 0;
  while (p < end) {
    const char* nl = (const char*)std::memchr(p, '\n', (size_t)(end - p));
    const char* e = nl ? nl : end;
    if (n < keep_first || !blank(p, e)) {
      rb.push_back(p);
      re.push_back(e);
    }
    ++n;
    p = nl ? nl + 1 : end;
  }
}

// split a record into up to maxn items (blank / tab / comma separated)
int items(const char* b, const char* e, const char** ib, const char** ie, int maxn) {
  int n = 0;
  while (b < e && n < maxn) {
    while (b < e && (*b == ' ' || *b == '\t' || *b == ',' || *b == '\r')) ++b;
    if (b >= e) break;
    const char* s = b;
    while (b < e && !(*b == ' ' || *b == '\t' || *b == ',' || *b == '\r')) ++b;
    ib[n] = s;
    ie[n] = b;
    ++n;
  }
  return n;
}

bool to_double(const char* b, const char* e, double& v) {
  char tmp[64];
  const size_t n = (size_t)(e - b);
  if (n == 0 || n >= sizeof(tmp)) return false;
  size_t j = 0;
  for (size_t i = 0; i < n; ++i) {
    char c = b[i];
    if (c == 'd' || c == 'D') c = 'e';
    if (i == 0 && c == '+') continue;   // from_chars takes no leading '+'
    tmp[j++] = c;
  }
  const auto r = std::from_chars(tmp, tmp + j, v);
  return r.ec == std::errc() && r.ptr == tmp + j;
}

bool to_int(const char* b, const char* e, int& v) {
  if (b < e && *b == '+') ++b;
  const auto r = std::from_chars(b, e, v);
  return r.ec == std::errc() && r.ptr == e;
}

int pool_size(int nthreads, size_t work) {
  int n = nthreads > 0 ? nthreads : (int)std::thread::hardware_concurrency();
  n = std::max(1, std::min(n, 64));
  return (int)std::min<size_t>((size_t)n, std::max<size_t>(work, 1));
}

// run f(i) for i in [0, n) on `threads` threads in contiguous chunks; returns false if any
// call returned false
template <class F>
bool parallel_for(size_t n, int threads, F&& f) {
  std::atomic<bool> ok{true};
  std::vector<std::thread> th;
  const size_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const size_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back([&, lo, hi] {
      for (size_t i = lo; i < hi && ok.load(std::memory_order_relaxed); ++i)
        if (!f(i)) ok = false;
    });
  }
  for (auto& t : th) t.join();
  return ok;
}

}  // namespace

int read_mmn(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell, double* m,
             int nthreads, std::string& err) {
  std::string buf;
  if (!load_file(path, buf)) {
    err = std::string("Error: Problem opening input file ") + path;
    return 6;
  }
  std::vector<const char*> rb, re;
  index_records(buf, 1, rb, re);
  const char* ib[8];
  const char* ie[8];
  int h[3];
  if (rb.size() < 2 || items(rb[1], re[1], ib, ie, 3) < 3 || !to_int(ib[0], ie[0], h[0]) ||
      !to_int(ib[1], ie[1], h[1]) || !to_int(ib[2], ie[2], h[2])) {
    err = std::string("Error: Problem reading input file ") + path;
    return 6;
  }
  if (h[0] != nb) {
    err = std::string(path) + " has not the right number of bands";
    return 6;
  }
  if (h[1] != nk) {
    err = std::string(path) + " has not the right number of k-points";
    return 6;
  }
  if (h[2] != nntot) {
    err = std::string(path) + " has not the right number of nearest neighbours";
    return 6;
  }
  const size_t nblk = (size_t)nk * nntot, per = 1 + (size_t)nb * nb;
  if (rb.size() < 2 + nblk * per) {
    err = std::string("Error: Problem reading input file ") + path;
    return 6;
  }
  const int threads = pool_size(nthreads, nblk);
  // pass 1: block headers -> destination slot k*nntot + nn
  std::vector<long long> dest(nblk, -1);
  std::atomic<int> bad{0};   // 1 parse, 2 not found, 3 more than one match
  parallel_for(nblk, threads, [&](size_t j) {
    const char* b[5];
    const char* e[5];
    const size_t r = 2 + j * per;
    int v[5];
    if (items(rb[r], re[r], b, e, 5) < 5) { bad = 1; return false; }
    for (int i = 0; i < 5; ++i)
      if (!to_int(b[i], e[i], v[i])) { bad = 1; return false; }
    const int k = v[0] - 1, k2 = v[1] - 1;
    if (k < 0 || k >= nk) { bad = 1; return false; }
    int nn = -1;
    for (int i = 0; i < nntot; ++i) {
      const size_t o = (size_t)k * nntot + i;
      if (nnlist[o] == k2 && nncell[3 * o] == v[2] && nncell[3 * o + 1] == v[3] && nncell[3 * o + 2] == v[4]) {
        if (nn >= 0) { bad = 3; return false; }
        nn = i;
      }
    }
    if (nn < 0) { bad = 2; return false; }
    dest[j] = (long long)k * nntot + nn;
    return true;
  });
  if (bad) {
    err = bad == 1 ? std::string("Error: Problem reading input file ") + path
          : bad == 2 ? std::string("Error reading ") + path + ": Neighbour not found"
                     : std::string("Error reading ") + path + ". More than one matching nearest neighbour found";
    return 6;
  }
  // a slot written twice keeps the later block (sequential-read semantics)
  std::vector<long long> last(nblk, -1);
  for (size_t j = 0; j < nblk; ++j) last[(size_t)dest[j]] = (long long)j;
  const size_t NN = (size_t)nb * nb;
  // pass 2: values, (m, n) with m fastest, straight into the destination block
  const bool ok = parallel_for(nblk, threads, [&](size_t j) {
    if (last[(size_t)dest[j]] != (long long)j) return true;
    double* out = m + 2 * (size_t)dest[j] * NN;
    const char* b[2];
    const char* e[2];
    for (size_t i = 0; i < NN; ++i) {
      const size_t r = 2 + j * per + 1 + i;
      if (items(rb[r], re[r], b, e, 2) < 2 || !to_double(b[0], e[0], out[2 * i]) ||
          !to_double(b[1], e[1], out[2 * i + 1]))
        return false;
    }
    return true;
  });
  if (!ok) {
    err = std::string("Error: Problem reading input file ") + path;
    return 6;
  }
  return 0;
}

int read_amn(const char* path, int nb, int nproj, int nk, double* a, int nthreads, std::string& err) {
  std::string buf;
  if (!load_file(path, buf)) {
    err = std::string("Error: Problem opening input file ") + path;
    return 6;
  }
  std::vector<const char*> rb, re;
  index_records(buf, 1, rb, re);
  const char* hb[3];
  const char* he[3];
  int h[3];
  if (rb.size() < 2 || items(rb[1], re[1], hb, he, 3) < 3 || !to_int(hb[0], he[0], h[0]) ||
      !to_int(hb[1], he[1], h[1]) || !to_int(hb[2], he[2], h[2])) {
    err = std::string("Error: Problem reading input file ") + path;
    return 6;
  }
  if (h[0] != nb) {
    err = std::string(path) + " has not the right number of bands";
    return 6;
  }
  if (h[1] != nk) {
    err = std::string(path) + " has not the right number of k-points";
    return 6;
  }
  if (h[2] != nproj) {
    err = std::string(path) + " has not the right number of projections";
    return 6;
  }
  const size_t nrec = (size_t)nb * nproj * nk;
  if (rb.size() < 2 + nrec) {
    err = std::string("Error: Problem reading input file ") + path;
    return 6;
  }
  const int threads = pool_size(nthreads, nrec / 4096 + 1);
  std::vector<long long> dest(nrec, -1);
  std::vector<double> val(2 * nrec);
  const bool ok = parallel_for(nrec, threads, [&](size_t j) {
    const char* b[5];
    const char* e[5];
    int v[3];
    const size_t r = 2 + j;
    if (items(rb[r], re[r], b, e, 5) < 5) return false;
    for (int i = 0; i < 3; ++i)
      if (!to_int(b[i], e[i], v[i])) return false;
    if (v[0] < 1 || v[0] > nb || v[1] < 1 || v[1] > nproj || v[2] < 1 || v[2] > nk) return false;
    if (!to_double(b[3], e[3], val[2 * j]) || !to_double(b[4], e[4], val[2 * j + 1])) return false;
    dest[j] = (long long)(v[0] - 1) + (long long)nb * ((v[1] - 1) + (long long)nproj * (v[2] - 1));
    return true;
  });
  if (!ok) {
    err = std::string("Error: Problem reading input file ") + path;
    return 6;
  }
  // in file order: later records overwrite earlier ones for the same (m, n, k)
  for (size_t j = 0; j < nrec; ++j) {
    a[2 * (size_t)dest[j]] = val[2 * j];
    a[2 * (size_t)dest[j] + 1] = val[2 * j + 1];
  }
  return 0;
}

int read_eig(const char* path, int nb, int nk, double* eig, std::string& err) {
  std::string buf;
  if (!load_file(path, buf)) {
    err = std::string("Error: Problem opening eigenvalue file ") + path;
    return 6;
  }
  std::vector<const char*> rb, re;
  index_records(buf, 0, rb, re);
  if (rb.size() < (size_t)nb * nk) {
    err = std::string("Error: Problem reading eigenvalue file ") + path;
    return 6;
  }
  size_t r = 0;
  for (int k = 0; k < nk; ++k)
    for (int n = 0; n < nb; ++n, ++r) {
      const char* b[3];
      const char* e[3];
      int i = 0, j = 0;
      if (items(rb[r], re[r], b, e, 3) < 3 || !to_int(b[0], e[0], i) || !to_int(b[1], e[1], j) ||
          !to_double(b[2], e[2], eig[(size_t)k * nb + n])) {
        err = std::string("Error: Problem reading eigenvalue file ") + path;
        return 6;
      }
      if (i != n + 1 || j != k + 1) {
        err = std::string("w90_wannier90_readwrite_read: mismatch in ") + path;
        return 6;
      }
    }
  return 0;
}

}  // namespace w90g
