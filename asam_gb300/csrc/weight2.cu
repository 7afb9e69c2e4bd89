// Cut-cell geometry files (<case>.Weight2), host code: the reader of
// ReadWeights (INIT/ReadWeights_Mod.f90:568-1330) and the writer of
// WriteWeightBlk (GRID/OutputWeightBlk_Mod.f90:501-670) for Cartesian grids.
//
// The file is Fortran list-directed text.  After the grid type and the block
// count, per block:
//   '#.... Block ib ....'; x0 y0 z0; nx and nx widths dx; ny, dy; nz, dz;
//   NrW_FacesYZ, then that many 'ix iy iz' / FU pairs (FU over ix0-1:ix1+1);
//   NrMP_FacesYZ, then 'ix iy iz' / 'xS yS zS' pairs; the same for FV (ZX)
//   and FW (XY); NrW_Cells, then 'ix iy iz' / VolC pairs;
//   'NrB_Cells Struct_Bound' then per boundary cell 'ix iy iz' / 'xS yS zS' /
//   'zRauh alb ee xFLS yFLS zFLS' followed, on the same READ, by the soil
//   types of every soil layer (Struct_Bound 4), the land class (5) or the
//   land class and the soil types (6).
// Every weight the file does not list keeps the reader's Cartesian default
// (ReadWeights_Mod.f90:633-640, 893-1000): full faces dy*dz, dx*dz, dx*dy;
// VolC = 1 on the halo's edges and corners, dx*dy*dz inside, and beside each
// face of the block dxLoc*dy*dz with dxLoc the width of the periodic
// partner's last cell (periodic side) or of the block's own first cell
// (outer wall).  The writer lists exactly the weights that differ from that
// default, each as the shortest decimal that reads back to the same double,
// so a written and re-read block is bit-identical.
//
// Each READ starts on a new line, takes values across lines as needed and
// drops the rest of its last line; values are separated by blanks or commas,
// 'r*c' repeats c r times, a '/' ends the READ, 'D' exponents and quoted
// strings are accepted.  Numbers are parsed and printed locale-independently
// (from_chars / to_chars: correctly rounded, shortest round-trip output).
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "context.h"

namespace {

constexpr int kStatusUnsupported = ASAM_UNSUPPORTED;

// roughness length per land class 0..9 (zrough, SOIL/SoilData_Mod.f90:104)
constexpr double kZrough[10] = {0.05, 1.0, 0.15, 1.0, 1.0, 1.0, 0.2, 0.5, 0.03, 0.01};
constexpr int kLandSea = 9;
constexpr double kZrauhSoil = 0.05;  // Struct_Bound 4 (ReadWeights_Mod.f90:1248)

int fail(int status, const std::string& msg) {
  asam::set_last_error(msg.c_str(), __FILE__, __LINE__);
  return status;
}

// ------------------------------------------------------------ list-directed READ
struct Tok {
  const char* s;
  int len;
};

class ListReader {
 public:
  ListReader(const char* b, const char* e) : p_(b), end_(e) {}

  // the next record, without its line end
  bool line(const char** s, const char** e) {
    if (p_ >= end_) return false;
    const char* q = (const char*)memchr(p_, '\n', size_t(end_ - p_));
    const char* le = q ? q : end_;
    *s = p_;
    *e = (le > p_ && le[-1] == '\r') ? le - 1 : le;
    p_ = q ? q + 1 : end_;
    return true;
  }

  const char* pos() const { return p_; }
  const char* end() const { return end_; }
  void seek(const char* p) { p_ = p; }

  // one READ of n values that must all stand on the current line (the
  // writers' layout); false, without an error text, when they do not
  bool read_line(Tok* out, int n) {
    const char* save = p_;
    const char *s, *e;
    if (!line(&s, &e)) return false;
    ListReader one(s, e);
    std::string err;
    if (!one.read(out, n, &err)) {
      p_ = save;
      return false;
    }
    return true;
  }

  // one READ of n values (n <= cap); the text of the error on failure
  bool read(Tok* out, int n, std::string* err) {
    int got = 0;
    while (got < n) {
      const char *s, *e;
      if (!line(&s, &e)) {
        *err = "unexpected end of file";
        return false;
      }
      const char* q = s;
      while (q < e) {
        while (q < e && (*q == ' ' || *q == '\t' || *q == ',')) ++q;
        if (q >= e) break;
        if (*q == '/') {
          *err = "list-directed read terminated early";
          return false;
        }
        Tok t;
        int rep = 1;
        if (*q == '\'' || *q == '"') {
          const char c = *q++;
          t.s = q;
          while (q < e && *q != c) ++q;
          t.len = int(q - t.s);
          if (q < e) ++q;
        } else {
          t.s = q;
          while (q < e && *q != ' ' && *q != '\t' && *q != ',' && *q != '/') ++q;
          t.len = int(q - t.s);
          // r*c: a repeat count of digits before the star
          const char* star = (const char*)memchr(t.s, '*', size_t(t.len));
          if (star && star > t.s) {
            bool digits = true;
            int r = 0;
            for (const char* c = t.s; c < star; ++c) {
              if (*c < '0' || *c > '9' || r > 100000000) {
                digits = false;
                break;
              }
              r = r * 10 + (*c - '0');
            }
            if (digits) {
              rep = r;
              t.len -= int(star + 1 - t.s);
              t.s = star + 1;
            }
          }
        }
        for (int k = 0; k < rep && got < n; ++k) out[got++] = t;
        if (got >= n) break;  // the rest of the record is dropped
      }
    }
    return true;
  }

 private:
  const char* p_;
  const char* end_;
};

bool to_int(const Tok& t, long long* v) {
  const char* c = t.s;
  const char* e = t.s + t.len;
  bool neg = false;
  if (c < e && (*c == '+' || *c == '-')) neg = *c++ == '-';
  if (c >= e) return false;
  long long r = 0;
  for (; c < e; ++c) {
    if (*c < '0' || *c > '9' || r > 1000000000000000LL) return false;
    r = r * 10 + (*c - '0');
  }
  *v = neg ? -r : r;
  return true;
}

// a real of a list-directed READ: Fortran's D (and Q) exponent letters, a
// leading '+'; parsed correctly rounded and locale-independent (from_chars)
bool to_real(const Tok& t, double* v) {
  char buf[80];
  if (t.len <= 0 || t.len >= int(sizeof(buf))) return false;
  int n = 0;
  for (int i = (t.s[0] == '+' ? 1 : 0); i < t.len; ++i) {
    const char c = t.s[i];
    buf[n++] = (c == 'D' || c == 'd' || c == 'Q' || c == 'q') ? 'E' : c;
  }
  if (n == 0) return false;
  const std::from_chars_result r = std::from_chars(buf, buf + n, *v);
  return r.ec == std::errc() && r.ptr == buf + n;
}

// ------------------------------------------------------------ block in memory
struct Block {
  int nx = 0, ny = 0, nz = 0;
  double origin[3] = {0, 0, 0};
  std::vector<double> dx, dy, dz, fu, fv, fw, volc;
  std::vector<int> mid_ijk[3];
  std::vector<double> mid_xs[3];
  int struct_bound = 0, nsoil = 0;
  std::vector<int> bijk, land, soil;
  std::vector<double> bxs, bsurf, normal, fl, dl;
};

// index of Fortran (ix,iy,iz) in the library's layout of each array, -1 outside:
// FU(ix,iy,iz) = fu[iz-1][iy-1][ix+1], FV = fv[iz-1][iy+1][ix-1],
// FW = fw[iz+1][iy-1][ix-1], VolC = volc[iz][iy][ix]
enum Arr { kFU = 0, kFV = 1, kFW = 2, kVol = 3 };
constexpr int kOff[4][3] = {{1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}, {0, 0, 0}};

void extents(int a, int nx, int ny, int nz, long long* ex, long long* ey, long long* ez) {
  switch (a) {
    case kFU: *ex = nx + 3, *ey = ny, *ez = nz; break;
    case kFV: *ex = nx, *ey = ny + 3, *ez = nz; break;
    case kFW: *ex = nx, *ey = ny, *ez = nz + 3; break;
    default: *ex = nx + 2, *ey = ny + 2, *ez = nz + 2;
  }
}

long long locate(int a, int nx, int ny, int nz, long long ix, long long iy, long long iz) {
  long long ex, ey, ez;
  extents(a, nx, ny, nz, &ex, &ey, &ez);
  const long long i = ix + kOff[a][0], j = iy + kOff[a][1], k = iz + kOff[a][2];
  if (i < 0 || j < 0 || k < 0 || i >= ex || j >= ey || k >= ez) return -1;
  return (k * ey + j) * ex + i;
}

int host_threads();

// work(t) for t = 0..n-1, t >= 1 on their own threads; a thread that cannot
// be started runs its part here, and every started thread is joined
template <typename F>
void run_parts(int n, F work) {
  std::vector<std::thread> pool;
  std::vector<int> inline_parts;
  for (int t = 1; t < n; ++t) {
    try {
      pool.emplace_back(work, t);
    } catch (...) {
      inline_parts.push_back(t);
    }
  }
  work(0);
  for (int t : inline_parts) work(t);
  for (auto& th : pool) th.join();
}

// f(k0, k1) over the slices of [0, n) on the host threads
template <typename F>
void for_slices(long long n, F f) {
  const int nth = n >= 16 ? host_threads() : 1;
  run_parts(nth, [&](int t) { f(n * t / nth, n * (t + 1) / nth); });
}

// The reader's Cartesian weights before the file's lists are applied
// (ReadWeights_Mod.f90:633-640, 893-1000); products in the reader's order.
void default_weights(const std::vector<double>& dx, const std::vector<double>& dy, const std::vector<double>& dz,
                     const int periodic[3], std::vector<double>* fu, std::vector<double>* fv,
                     std::vector<double>* fw, std::vector<double>* volc) {
  const long long nx = (long long)dx.size(), ny = (long long)dy.size(), nz = (long long)dz.size();
  // every element is written below (the halo edges and corners of VolC = 1)
  fu->resize(size_t((nx + 3) * ny * nz));
  fv->resize(size_t(nx * (ny + 3) * nz));
  fw->resize(size_t(nx * ny * (nz + 3)));
  volc->resize(size_t((nx + 2) * (ny + 2) * (nz + 2)));
  for_slices(nz, [&](long long k0, long long k1) {
    for (long long k = k0; k < k1; ++k)
      for (long long j = 0; j < ny; ++j) {
        const double a = dz[k] * dy[j];
        double* r = fu->data() + (k * ny + j) * (nx + 3);
        for (long long i = 0; i < nx + 3; ++i) r[i] = a;
      }
    for (long long k = k0; k < k1; ++k)
      for (long long j = 0; j < ny + 3; ++j) {
        double* r = fv->data() + (k * (ny + 3) + j) * nx;
        for (long long i = 0; i < nx; ++i) r[i] = dz[k] * dx[i];
      }
  });
  for_slices(nz + 3, [&](long long k0, long long k1) {
    for (long long k = k0; k < k1; ++k)
      for (long long j = 0; j < ny; ++j) {
        double* r = fw->data() + (k * ny + j) * nx;
        for (long long i = 0; i < nx; ++i) r[i] = dy[j] * dx[i];
      }
  });
  const long long sx = nx + 2, sy = ny + 2;
  double* v = volc->data();
  auto at = [&](long long k, long long j, long long i) -> double& { return v[(k * sy + j) * sx + i]; };
  for_slices(nz + 2, [&](long long k0, long long k1) {
    for (long long k = k0; k < k1; ++k) {
      double* pl = v + k * sy * sx;
      std::fill(pl, pl + sy * sx, 1.0);
      if (k < 1 || k > nz) continue;
      for (long long j = 1; j <= ny; ++j)
        for (long long i = 1; i <= nx; ++i) at(k, j, i) = dx[i - 1] * dy[j - 1] * dz[k - 1];
    }
  });
  const double dxw = periodic[0] ? dx[nx - 1] : dx[0], dxe = periodic[0] ? dx[0] : dx[nx - 1];
  const double dys = periodic[1] ? dy[ny - 1] : dy[0], dyn = periodic[1] ? dy[0] : dy[ny - 1];
  const double dzb = periodic[2] ? dz[nz - 1] : dz[0], dzt = periodic[2] ? dz[0] : dz[nz - 1];
  for (long long k = 1; k <= nz; ++k)
    for (long long j = 1; j <= ny; ++j) {
      at(k, j, 0) = dxw * dy[j - 1] * dz[k - 1];
      at(k, j, nx + 1) = dxe * dy[j - 1] * dz[k - 1];
    }
  for (long long k = 1; k <= nz; ++k)
    for (long long i = 1; i <= nx; ++i) {
      at(k, 0, i) = dys * dx[i - 1] * dz[k - 1];
      at(k, ny + 1, i) = dyn * dx[i - 1] * dz[k - 1];
    }
  for (long long j = 1; j <= ny; ++j)
    for (long long i = 1; i <= nx; ++i) {  // dx(jx)*dy(jy)*dzLoc (ReadWeights_Mod.f90:962-987)
      at(0, j, i) = dx[i - 1] * dy[j - 1] * dzb;
      at(nz + 1, j, i) = dx[i - 1] * dy[j - 1] * dzt;
    }
}

// Surface normal, area and wall distance of each boundary cell
// (ReadWeights_Mod.f90:1283-1319): the area differences of opposite faces,
// a pair of closed opposite faces counting as twice the full face.
void normals(Block& B) {
  const size_t n = B.land.size();
  B.normal.resize(3 * n);
  B.fl.resize(n);
  B.dl.resize(n);
  const int nx = B.nx, ny = B.ny, nz = B.nz;
  for (size_t q = 0; q < n; ++q) {
    const long long i = B.bijk[3 * q], j = B.bijk[3 * q + 1], k = B.bijk[3 * q + 2];
    const double fuR = B.fu[size_t(locate(kFU, nx, ny, nz, i, j, k))];
    const double fuL = B.fu[size_t(locate(kFU, nx, ny, nz, i - 1, j, k))];
    const double fvR = B.fv[size_t(locate(kFV, nx, ny, nz, i, j, k))];
    const double fvL = B.fv[size_t(locate(kFV, nx, ny, nz, i, j - 1, k))];
    const double fwR = B.fw[size_t(locate(kFW, nx, ny, nz, i, j, k))];
    const double fwL = B.fw[size_t(locate(kFW, nx, ny, nz, i, j, k - 1))];
    const double ddx = B.dx[size_t(i - 1)], ddy = B.dy[size_t(j - 1)], ddz = B.dz[size_t(k - 1)];
    const double n1 = (fuR == 0.0 && fuL == 0.0) ? ddy * ddz * 2.0 : fuR - fuL;
    const double n2 = (fvR == 0.0 && fvL == 0.0) ? ddx * ddz * 2.0 : fvR - fvL;
    const double n3 = (fwR == 0.0 && fwL == 0.0) ? ddx * ddy * 2.0 : fwR - fwL;
    double fl = std::sqrt(n1 * n1 + n2 * n2 + n3 * n3);
    double m1 = 0.0, m2 = 0.0, m3 = 1.0;
    if (fl > 0.0) {
      m1 = n1 / fl, m2 = n2 / fl, m3 = n3 / fl;
    } else {
      fl = 1e-10;
    }
    B.normal[3 * q] = m1, B.normal[3 * q + 1] = m2, B.normal[3 * q + 2] = m3;
    B.fl[q] = fl;
    const double a = m1 * ddx, b = m2 * ddy, c = m3 * ddz;
    B.dl[q] = 0.5 * std::sqrt(a * a + b * b + c * c);
  }
}

int host_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(hw, 16u));
}

// The cnt pairs of READs 'ix iy iz' / value after a weight count, parsed by
// several threads when every READ finds its values on its own line (the
// layout both writers produce): the 2*cnt lines are cut into chunks at pair
// boundaries, each thread parses its chunk into (index, value) entries, and
// the entries are applied in file order (a repeated index keeps the last
// value, as the sequential READs do).  False leaves the reader where it was
// and the caller parses the pairs one READ at a time, which also gives the
// exact error of a malformed pair.
bool pairs_parallel(ListReader& rd, long long cnt, int a, int nx, int ny, int nz, double* dst) {
  const int nth = host_threads();
  if (cnt < (1 << 16) || nth < 2) return false;
  const char* start = rd.pos();
  const long long lines = 2 * cnt;
  const long long per = ((lines / nth) + 1) & ~1LL;  // even: chunks begin at a pair
  std::vector<const char*> cut{start};
  ListReader scan(start, rd.end());
  for (long long L = 0; L < lines; ++L) {
    const char *s, *e;
    if (!scan.line(&s, &e)) return false;
    if ((L + 1) % per == 0 && L + 1 < lines) cut.push_back(scan.pos());
  }
  const char* q = scan.pos();
  cut.push_back(q);
  const int nch = (int)cut.size() - 1;
  std::vector<std::vector<std::pair<long long, double>>> got(nch);
  std::vector<char> ok(nch, 1);
  auto parse_chunk = [&](int t) {
    ListReader r(cut[t], cut[t + 1]);
    Tok tk[3];
    auto& out = got[t];
    out.reserve(size_t(per / 2 + 1));
    while (r.pos() < cut[t + 1]) {
      long long v[3];
      double w;
      if (!r.read_line(tk, 3) || !to_int(tk[0], &v[0]) || !to_int(tk[1], &v[1]) || !to_int(tk[2], &v[2]) ||
          !r.read_line(tk, 1) || !to_real(tk[0], &w)) {
        ok[t] = 0;
        return;
      }
      const long long at = locate(a, nx, ny, nz, v[0], v[1], v[2]);
      if (at < 0) {
        ok[t] = 0;
        return;
      }
      out.emplace_back(at, w);
    }
  };
  auto work = [&](int t) noexcept {  // an allocation that fails sends the list to the sequential parse
    try {
      parse_chunk(t);
    } catch (...) {
      ok[t] = 0;
    }
  };
  run_parts(nch, work);
  long long n = 0;
  for (int t = 0; t < nch; ++t) {
    if (!ok[t]) return false;
    n += (long long)got[t].size();
  }
  if (n != cnt) return false;
  for (int t = 0; t < nch; ++t)
    for (const auto& e : got[t]) dst[e.first] = e.second;
  rd.seek(q);
  return true;
}

int parse(const char* buf, size_t size, int ib, const asam_weight2_options& o, Block& B) {
  ListReader rd(buf, buf + size);
  Tok t[64];
  std::string err;
  auto io = [&](const std::string& m) { return fail(ASAM_IO_ERROR, "Weight2: " + m); };
#define RD(n)                          \
  do {                                 \
    if (!rd.read(t, (n), &err)) return io(err); \
  } while (0)
  auto num_i = [&](int k, long long* v) { return to_int(t[k], v); };
  auto num_r = [&](int k, double* v) { return to_real(t[k], v); };
  RD(1);
  const std::string grid(t[0].s, size_t(t[0].len));
  if (grid != "Cart")
    return fail(kStatusUnsupported, "Weight2 reader: grid type '" + grid + "' (Cartesian grids only)");
  long long nb = 0;
  RD(1);
  if (!num_i(0, &nb)) return io("bad block count");
  if (ib < 1 || ib > nb) return io("block " + std::to_string(ib) + " of " + std::to_string(nb));
  // S: DO ... READ(InputUnit,'(a300)') Line until '#.... Block ib' (ReadWeights_Mod.f90:581-585)
  static const char kTag[] = "#.... Block";
  for (;;) {
    const char *s, *e;
    if (!rd.line(&s, &e)) return io("unexpected end of file");
    const char* at = std::search(s, e, kTag, kTag + sizeof(kTag) - 1);
    if (at == e) continue;
    ListReader sub(at + sizeof(kTag) - 1, e);
    Tok b;
    long long v;
    if (sub.read(&b, 1, &err) && to_int(b, &v) && v == ib) break;
  }
  RD(3);
  for (int a = 0; a < 3; ++a)
    if (!num_r(a, &B.origin[a])) return io("bad origin");
  std::vector<double>* widths[3] = {&B.dx, &B.dy, &B.dz};
  int* ns[3] = {&B.nx, &B.ny, &B.nz};
  for (int a = 0; a < 3; ++a) {
    long long n = 0;
    RD(1);
    if (!num_i(0, &n) || n < 1 || n > (1LL << 24)) return io("bad cell count");
    if (o.expect[a] > 0 && n != o.expect[a])
      return io(std::string("Error WeightFile (n") + "xyz"[a] + ")");
    *ns[a] = int(n);
    widths[a]->resize(size_t(n));
    for (long long i = 0; i < n; ++i) {
      RD(1);
      if (!num_r(0, &(*widths[a])[size_t(i)])) return io("bad cell width");
    }
  }
  const int nx = B.nx, ny = B.ny, nz = B.nz;
  default_weights(B.dx, B.dy, B.dz, o.periodic, &B.fu, &B.fv, &B.fw, &B.volc);
  std::vector<double>* arrs[4] = {&B.fu, &B.fv, &B.fw, &B.volc};
  static const char* kName[4] = {"FU", "FV", "FW", "VolC"};
  auto weights = [&](int a) -> int {
    long long cnt = 0;
    RD(1);
    if (!num_i(0, &cnt) || cnt < 0) return io("bad entry count");
    double* dst = arrs[a]->data();
    if (pairs_parallel(rd, cnt, a, nx, ny, nz, dst)) return ASAM_OK;
    for (long long q = 0; q < cnt; ++q) {
      long long ix, iy, iz;
      double v;
      RD(3);
      if (!num_i(0, &ix) || !num_i(1, &iy) || !num_i(2, &iz)) return io("bad index");
      RD(1);
      if (!num_r(0, &v)) return io("bad weight");
      const long long at = locate(a, nx, ny, nz, ix, iy, iz);
      if (at < 0) return io(std::string(kName[a]) + " index outside the block");
      dst[at] = v;
    }
    return ASAM_OK;
  };
  for (int a = 0; a < 3; ++a) {
    int st = weights(a);
    if (st != ASAM_OK) return st;
    long long cnt = 0;
    RD(1);
    if (!num_i(0, &cnt) || cnt < 0) return io("bad midpoint count");
    for (long long q = 0; q < cnt; ++q) {
      long long v[3];
      double x[3];
      RD(3);
      for (int c = 0; c < 3; ++c)
        if (!num_i(c, &v[c]) || v[c] < INT32_MIN || v[c] > INT32_MAX) return io("bad index");
      RD(3);
      for (int c = 0; c < 3; ++c)
        if (!num_r(c, &x[c])) return io("bad midpoint");
      for (int c = 0; c < 3; ++c) B.mid_ijk[a].push_back(int(v[c])), B.mid_xs[a].push_back(x[c]);
    }
  }
  {
    int st = weights(kVol);
    if (st != ASAM_OK) return st;
  }
  // NumBoundCell, Str_Read, nr_structbound (ReadWeights_Mod.f90:1217)
  long long nbc = 0, sb = 0;
  RD(3);
  if (!num_i(0, &nbc) || nbc < 0 || !num_i(2, &sb)) return io("bad boundary-cell header");
  if (sb < 0 || sb > 6) return fail(kStatusUnsupported, "Weight2 reader: Struct_Bound " + std::to_string(sb));
  const int nsoil = o.nr_soil_layers;
  const int ntail = sb == 4 ? nsoil : sb == 5 ? 1 : sb == 6 ? 1 + nsoil : 0;
  if (6 + ntail > int(sizeof(t) / sizeof(t[0]))) return fail(ASAM_BAD_ARG, "Weight2: too many soil layers");
  B.struct_bound = int(sb);
  B.nsoil = nsoil;
  for (long long q = 0; q < nbc; ++q) {
    long long v[3];
    RD(3);
    for (int c = 0; c < 3; ++c)
      if (!num_i(c, &v[c])) return io("bad boundary-cell index");
    if (v[0] < 1 || v[0] > nx || v[1] < 1 || v[1] > ny || v[2] < 1 || v[2] > nz)
      return io("boundary cell outside the block");
    for (int c = 0; c < 3; ++c) B.bijk.push_back(int(v[c]));
    RD(3);
    for (int c = 0; c < 3; ++c) {
      double x;
      if (!num_r(c, &x)) return io("bad boundary-cell midpoint");
      B.bxs.push_back(x);
    }
    RD(6 + ntail);
    double s[6];
    for (int c = 0; c < 6; ++c)
      if (!num_r(c, &s[c])) return io("bad surface data");
    long long tail[64];
    for (int c = 0; c < ntail; ++c)
      if (!num_i(6 + c, &tail[c])) return io("bad soil or land class");
    // ReadWeights_Mod.f90:1236-1279: the roughness and the classes each Struct_Bound implies
    int land = o.land_class_def;
    const size_t s0 = B.soil.size();
    B.soil.resize(s0 + size_t(nsoil), 0);
    int* soil = B.soil.data() + s0;
    if (sb == 4) {
      for (int c = 0; c < nsoil; ++c) soil[c] = int(tail[c]);
      s[0] = kZrauhSoil;
    } else if (sb == 5) {
      land = kLandSea;  // only the sea class is read
      s[0] = kZrough[land];
    } else if (sb == 6) {
      if (tail[0] < 0 || tail[0] > 9) return io("land class outside 0-9");
      land = int(tail[0]);
      for (int c = 0; c < nsoil; ++c) soil[c] = int(tail[1 + c]);
      s[0] = kZrough[land];
    } else if (nsoil > 0) {
      soil[nsoil - 1] = 5;
    }
    B.land.push_back(land);
    for (int c = 0; c < 6; ++c) B.bsurf.push_back(s[c]);
  }
#undef RD
  if (o.real_island) {  // a boundary cell of full volume is an island in the sea
    for (size_t q = 0; q < B.land.size(); ++q) {
      const long long i = B.bijk[3 * q], j = B.bijk[3 * q + 1], k = B.bijk[3 * q + 2];
      const double vol = B.volc[size_t(locate(kVol, nx, ny, nz, i, j, k))];
      if (vol >= B.dx[size_t(i - 1)] * B.dy[size_t(j - 1)] * B.dz[size_t(k - 1)] * 0.9999) B.land[q] = kLandSea;
    }
  }
  normals(B);
  return ASAM_OK;
}

// ------------------------------------------------------------ writer
void put_int(std::string& o, long long v, int width = 0) {
  char tmp[32];
  const char* e = std::to_chars(tmp, tmp + sizeof(tmp), v).ptr;
  for (int pad = width - int(e - tmp); pad > 0; --pad) o.push_back(' ');
  o.append(tmp, size_t(e - tmp));
}
// the shortest decimal that reads back to the same double (to_chars), with
// a decimal point kept on integral values
void put_real(std::string& o, double v) {
  char tmp[40];
  char* e = std::to_chars(tmp, tmp + sizeof(tmp) - 2, v).ptr;
  bool plain = true;
  for (const char* c = tmp; c < e; ++c)
    if (*c == '.' || *c == 'e' || *c == 'n' || *c == 'i') plain = false;
  if (plain) *e++ = '.', *e++ = '0';
  o.append(tmp, size_t(e - tmp));
}

class Out {
 public:
  explicit Out(FILE* f) : f_(f) { buf_.reserve(kFlush + 4096); }
  void put(const char* s, size_t n) {
    buf_.append(s, n);
    if (buf_.size() >= kFlush) flush();
  }
  void put(const char* s) { put(s, strlen(s)); }
  void put(const std::string& s) { put(s.data(), s.size()); }
  void integer(long long v, int width = 0) {
    put_int(buf_, v, width);
    if (buf_.size() >= kFlush) flush();
  }
  void real(double v) {
    put_real(buf_, v);
    if (buf_.size() >= kFlush) flush();
  }
  // a large finished piece: flushed, then written as it is
  void put_large(const std::string& t) {
    flush();
    if (!t.empty() && fwrite(t.data(), 1, t.size(), f_) != t.size()) ok_ = false;
  }
  bool flush() {
    if (!buf_.empty() && fwrite(buf_.data(), 1, buf_.size(), f_) != buf_.size()) ok_ = false;
    buf_.clear();
    return ok_;
  }
  bool ok() const { return ok_; }

 private:
  static constexpr size_t kFlush = size_t(8) << 20;
  FILE* f_;
  std::string buf_;
  bool ok_ = true;
};

int check_block(const asam_weight2_block& b, int ib) {
  const std::string w = "asam_weight2_write: block " + std::to_string(ib) + ": ";
  if (b.nx < 1 || b.ny < 1 || b.nz < 1) return fail(ASAM_BAD_ARG, w + "empty block");
  if (!b.dx || !b.dy || !b.dz || !b.fu || !b.fv || !b.fw || !b.volc) return fail(ASAM_BAD_ARG, w + "missing array");
  if (b.struct_bound < 0 || b.struct_bound > 6) return fail(ASAM_BAD_ARG, w + "Struct_Bound outside 0-6");
  if (b.nbound < 0 || b.nsoil < 0) return fail(ASAM_BAD_ARG, w + "negative count");
  if (b.nbound > 0 && (!b.bound_ijk || !b.bound_xs || !b.bound_surf))
    return fail(ASAM_BAD_ARG, w + "missing boundary-cell array");
  if (b.nbound > 0 && (b.struct_bound == 5 || b.struct_bound == 6) && !b.land_class)
    return fail(ASAM_BAD_ARG, w + "missing land classes");
  if (b.nbound > 0 && b.nsoil > 0 && (b.struct_bound == 4 || b.struct_bound == 6) && !b.soil_type)
    return fail(ASAM_BAD_ARG, w + "missing soil types");
  for (int a = 0; a < 3; ++a)
    if (b.nmid[a] < 0 || (b.nmid[a] > 0 && (!b.mid_ijk[a] || !b.mid_xs[a])))
      return fail(ASAM_BAD_ARG, w + "missing cut-face midpoints");
  const void* ptrs[] = {b.dx, b.dy, b.dz, b.fu, b.fv, b.fw, b.volc, b.bound_ijk, b.bound_xs, b.bound_surf,
                        b.land_class, b.soil_type, b.mid_ijk[0], b.mid_ijk[1], b.mid_ijk[2], b.mid_xs[0],
                        b.mid_xs[1], b.mid_xs[2], b.normal, b.fl, b.dl};
  for (const void* p : ptrs)
    if (asam::device_array(p)) return fail(ASAM_BAD_ARG, w + "device array (the file routines take host arrays)");
  return ASAM_OK;
}

void write_block(Out& out, const asam_weight2_block& b, int ib, const int periodic[3]) {
  std::vector<double> dx(b.dx, b.dx + b.nx), dy(b.dy, b.dy + b.ny), dz(b.dz, b.dz + b.nz);
  out.put(" #.... Block ");
  out.integer(ib);
  out.put(" .....................................................\n ");
  for (int a = 0; a < 3; ++a) {
    if (a) out.put(" ");
    out.real(b.origin[a]);
  }
  out.put("\n");
  const int n3[3] = {b.nx, b.ny, b.nz};
  const double* w3[3] = {b.dx, b.dy, b.dz};
  for (int a = 0; a < 3; ++a) {
    out.put(" ");
    out.integer(n3[a]);
    out.put("\n");
    for (int i = 0; i < n3[a]; ++i) {
      out.put(" ");
      out.real(w3[a][i]);
      out.put("\n");
    }
  }
  std::vector<double> ref[4];
  default_weights(dx, dy, dz, periodic, &ref[0], &ref[1], &ref[2], &ref[3]);
  const double* arr[4] = {b.fu, b.fv, b.fw, b.volc};
  static const char* kCount[4] = {"NrW_FacesYZ", "NrW_FacesZX", "NrW_FacesXY", "NrW_Cells"};
  static const char* kMid[3] = {"NrMP_FacesYZ", "NrMP_FacesZX", "NrMP_FacesXY"};
  // the weights that differ from the defaults, formatted by several threads
  // over slices of the array and written in index order
  auto entries = [&](int a) {
    long long ex, ey, ez;
    extents(a, b.nx, b.ny, b.nz, &ex, &ey, &ez);
    const double* v = arr[a];
    const double* r = ref[a].data();
    const long long n = ex * ey * ez;
    const int nth = n >= (1 << 18) ? host_threads() : 1;
    std::vector<std::string> text(nth);
    std::vector<long long> cnt(nth, 0);
    std::vector<char> fine(nth, 1);
    auto format = [&](int t) {
      const long long q0 = n * t / nth, q1 = n * (t + 1) / nth;
      std::string& o = text[t];
      for (long long q = q0; q < q1; ++q) {
        if (!(v[q] != r[q])) continue;
        const long long i = q % ex, j = (q / ex) % ey, k = q / (ex * ey);
        o.push_back(' ');
        put_int(o, i - kOff[a][0]);
        o.push_back(' ');
        put_int(o, j - kOff[a][1]);
        o.push_back(' ');
        put_int(o, k - kOff[a][2]);
        o.append("\n ");
        put_real(o, v[q]);
        o.push_back('\n');
        ++cnt[t];
      }
    };
    auto work = [&](int t) noexcept {
      try {
        format(t);
      } catch (...) {
        fine[t] = 0;
      }
    };
    run_parts(nth, work);
    for (char f : fine)
      if (!f) throw std::bad_alloc();
    long long total = 0;
    for (long long c : cnt) total += c;
    out.put(" ");
    out.integer(total);
    out.put(a == kVol ? "    " : "   ");
    out.put(kCount[a]);
    out.put("\n");
    for (auto& t : text) {
      out.put_large(t);
      std::string().swap(t);
    }
  };
  for (int a = 0; a < 3; ++a) {
    entries(a);
    out.put(" ");
    out.integer(b.nmid[a]);
    out.put("   ");
    out.put(kMid[a]);
    out.put("\n");
    for (int q = 0; q < b.nmid[a]; ++q) {
      const int* m = b.mid_ijk[a] + 3 * q;
      const double* x = b.mid_xs[a] + 3 * q;
      out.put(" ");
      out.integer(m[0]);
      out.put(" ");
      out.integer(m[1]);
      out.put(" ");
      out.integer(m[2]);
      out.put("\n ");
      out.real(x[0]);
      out.put(" ");
      out.real(x[1]);
      out.put(" ");
      out.real(x[2]);
      out.put("\n");
    }
  }
  entries(kVol);
  const int sb = b.struct_bound;
  const int nsoil = (sb == 4 || sb == 6) ? b.nsoil : 0;
  out.integer(b.nbound, 12);
  out.put("      NrB_Cells");
  out.integer(sb, 6);
  out.put("   Struct_Bound");
  out.integer(nsoil, 6);
  out.put("  Nr_SoilLayers\n");
  for (int q = 0; q < b.nbound; ++q) {
    const int* m = b.bound_ijk + 3 * q;
    const double* x = b.bound_xs + 3 * q;
    const double* s = b.bound_surf + 6 * q;
    out.put(" ");
    out.integer(m[0]);
    out.put(" ");
    out.integer(m[1]);
    out.put(" ");
    out.integer(m[2]);
    out.put("\n");
    for (int c = 0; c < 3; ++c) {
      out.put(" ");
      out.real(x[c]);
    }
    out.put("\n");
    for (int c = 0; c < 6; ++c) {
      out.put(" ");
      out.real(s[c]);
    }
    if (sb == 5 || sb == 6) {
      out.put(" ");
      out.integer(b.land_class[q]);
    }
    for (int c = 0; c < nsoil; ++c) {
      out.put(" ");
      out.integer(b.soil_type[size_t(q) * size_t(nsoil) + size_t(c)]);
    }
    out.put("\n");
  }
}

}  // namespace

struct asam_weight2_file {
  Block b;
};

extern "C" {

int asam_weight2_open(const char* path, int ib, const asam_weight2_options* opt, asam_weight2_file** out,
                      asam_weight2_block* info) {
  if (!path || !opt || !out || !info) return fail(ASAM_BAD_ARG, "asam_weight2_open: null argument");
  *out = nullptr;
  if (opt->nr_soil_layers < 0 || opt->nr_soil_layers > 57)
    return fail(ASAM_BAD_ARG, "asam_weight2_open: nr_soil_layers outside 0-57");
  if (opt->land_class_def < 0 || opt->land_class_def > 9)
    return fail(ASAM_BAD_ARG, "asam_weight2_open: land_class_def outside 0-9");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(ASAM_IO_ERROR, std::string("Weight2: cannot open ") + path);
  std::vector<char> text;
  long sz = -1;
  if (fseek(f, 0, SEEK_END) == 0) {
    sz = ftell(f);
    fseek(f, 0, SEEK_SET);
  }
  bool bad = false;
  try {
    if (sz >= 0) {  // one read into a buffer of the file's size
      text.resize(size_t(sz));
      bad = fread(text.data(), 1, text.size(), f) != text.size();
    } else {  // not seekable: in chunks
      char chunk[1 << 16];
      size_t got;
      while ((got = fread(chunk, 1, sizeof(chunk), f)) > 0) text.insert(text.end(), chunk, chunk + got);
      bad = ferror(f) != 0;
    }
  } catch (const std::exception&) {
    bad = true;
  }
  fclose(f);
  if (bad) return fail(ASAM_IO_ERROR, std::string("Weight2: read error on ") + path);
  asam_weight2_file* h = nullptr;
  int st;
  try {
    h = new asam_weight2_file();
    st = parse(text.data(), text.size(), ib, *opt, h->b);
  } catch (const std::exception& e) {  // out of host memory: nothing crosses the C boundary
    st = fail(ASAM_IO_ERROR, std::string("Weight2: ") + e.what());
  }
  if (st != ASAM_OK) {
    delete h;
    return st;
  }
  const Block& B = h->b;
  memset(info, 0, sizeof(*info));
  info->nx = B.nx, info->ny = B.ny, info->nz = B.nz;
  for (int a = 0; a < 3; ++a) info->origin[a] = B.origin[a], info->nmid[a] = int(B.mid_xs[a].size() / 3);
  info->nbound = int(B.land.size());
  info->struct_bound = B.struct_bound;
  info->nsoil = B.nsoil;
  *out = h;
  return ASAM_OK;
}

int asam_weight2_fetch(const asam_weight2_file* h, const asam_weight2_block* dst) {
  if (!h || !dst) return fail(ASAM_BAD_ARG, "asam_weight2_fetch: null argument");
  const Block& B = h->b;
  const void* ptrs[] = {dst->dx, dst->dy, dst->dz, dst->fu, dst->fv, dst->fw, dst->volc, dst->bound_ijk,
                        dst->bound_xs, dst->bound_surf, dst->land_class, dst->soil_type, dst->mid_ijk[0],
                        dst->mid_ijk[1], dst->mid_ijk[2], dst->mid_xs[0], dst->mid_xs[1], dst->mid_xs[2],
                        dst->normal, dst->fl, dst->dl};
  for (const void* p : ptrs)
    if (asam::device_array(p))
      return fail(ASAM_BAD_ARG, "asam_weight2_fetch: device array (the file routines take host arrays)");
  auto copy = [](void* to, const auto& v) {
    if (to && !v.empty()) memcpy(to, v.data(), v.size() * sizeof(v[0]));
  };
  copy(dst->dx, B.dx), copy(dst->dy, B.dy), copy(dst->dz, B.dz);
  copy(dst->fu, B.fu), copy(dst->fv, B.fv), copy(dst->fw, B.fw), copy(dst->volc, B.volc);
  for (int a = 0; a < 3; ++a) copy(dst->mid_ijk[a], B.mid_ijk[a]), copy(dst->mid_xs[a], B.mid_xs[a]);
  copy(dst->bound_ijk, B.bijk), copy(dst->bound_xs, B.bxs), copy(dst->bound_surf, B.bsurf);
  copy(dst->land_class, B.land), copy(dst->soil_type, B.soil);
  copy(dst->normal, B.normal), copy(dst->fl, B.fl), copy(dst->dl, B.dl);
  return ASAM_OK;
}

void asam_weight2_close(asam_weight2_file* h) { delete h; }

int asam_weight2_write(const char* path, int nblock, const asam_weight2_block* blocks, const int periodic[3]) {
  if (!path || nblock < 1 || !blocks || !periodic) return fail(ASAM_BAD_ARG, "asam_weight2_write: bad argument");
  for (int ib = 0; ib < nblock; ++ib) {
    const int st = check_block(blocks[ib], ib + 1);
    if (st != ASAM_OK) return st;
  }
  FILE* f = fopen(path, "wb");
  if (!f) return fail(ASAM_IO_ERROR, std::string("Weight2: cannot create ") + path);
  bool ok;
  try {
    Out out(f);
    out.put(" Cart\n ");
    out.integer(nblock);
    out.put("  ! Number of blocks\n");
    for (int ib = 0; ib < nblock; ++ib) write_block(out, blocks[ib], ib + 1, periodic);
    ok = out.flush();
  } catch (const std::exception& e) {  // out of host memory
    fclose(f);
    return fail(ASAM_IO_ERROR, std::string("Weight2: ") + e.what());
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) return fail(ASAM_IO_ERROR, std::string("Weight2: write error on ") + path);
  return ASAM_OK;
}

}  // extern "C"
