// lh_io.cpp -- the reference's file formats for fields, statistics and spectra.
//
// All files are Fortran sequential unformatted: every record is framed by a
// 4-byte little-endian length before and after it (gfortran's default).
//   restart fields  read by read_in (start.f90:1786-2235), written by the
//                   reference's record_out (FOU3D.f90, missing): per field a
//                   file <dir>/<u1|u2|u3|p><name>; records: header
//                   (t, Re, alp, bet, mpgx, nband, iter, 88 zero ints), N(4,0:4),
//                   one record read_in skips (here: the field's y coordinates),
//                   then one record per y plane of the field's grid:
//                   jin, band, nx, nz, y(jin), buffSR(N1+2, N2) -- the packed
//                   x-half-spectrum (re, im pairs) of the plane's N2 z modes.
//   statistics      write_stats (stats.f90:355-410)
//   spectra         recvwrspec (spectra.f90:109-180)
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/littleharsh.h"

namespace {

struct Writer {
  FILE* f = nullptr;
  bool ok = true;
  explicit Writer(const char* path) { f = std::fopen(path, "wb"); ok = f != nullptr; }
  ~Writer() { if (f) std::fclose(f); }
  // one record made of consecutive pieces
  void record(const std::vector<std::pair<const void*, size_t>>& parts) {
    if (!ok) return;
    size_t n = 0;
    for (auto& p : parts) n += p.second;
    if (n > 0x7fffffffu) { ok = false; return; }
    const uint32_t len = (uint32_t)n;
    ok = ok && std::fwrite(&len, 4, 1, f) == 1;
    for (auto& p : parts)
      if (p.second) ok = ok && std::fwrite(p.first, 1, p.second, f) == p.second;
    ok = ok && std::fwrite(&len, 4, 1, f) == 1;
  }
};

struct Reader {
  FILE* f = nullptr;
  bool ok = true;
  explicit Reader(const char* path) { f = std::fopen(path, "rb"); ok = f != nullptr; }
  ~Reader() { if (f) std::fclose(f); }
  // next record into buf (resized); returns its length or -1
  long record(std::vector<unsigned char>& buf) {
    if (!ok) return -1;
    uint32_t a = 0, b = 0;
    if (std::fread(&a, 4, 1, f) != 1) { ok = false; return -1; }
    buf.resize(a);
    if (a && std::fread(buf.data(), 1, a, f) != a) { ok = false; return -1; }
    if (std::fread(&b, 4, 1, f) != 1 || a != b) { ok = false; return -1; }
    return (long)a;
  }
};

struct Header {
  double t, Re, alp, bet, mpgx;
  int32_t nband, iter, dumm[88];
};

std::vector<std::pair<const void*, size_t>> header_parts(const Header& h) {
  return {{&h.t, 8}, {&h.Re, 8}, {&h.alp, 8}, {&h.bet, 8}, {&h.mpgx, 8}, {&h.nband, 4}, {&h.iter, 4},
          {h.dumm, 4 * 88}};
}

}  // namespace

namespace lh {
void set_handle_error(lh_handle* h, const char* msg);  // lh_capi.cu
}

namespace {

thread_local lh_handle* g_cur = nullptr;  // handle whose call is being served (for error messages)

int io_fail(int code, const std::string& msg) {
  lh::set_handle_error(g_cur, msg.c_str());
  return code;
}

// Grid sizes from the handle: nkx, nz, ngx, ngz, nyu, nyv, nyp, ju0, jv0, jp0, ...
struct Sz {
  int nkx, nz, ngx, ngz, nyu, nyv, nyp, ju0, jv0, jp0;
};

int sizes(lh_handle* h, Sz* s) {
  int32_t o[12];
  int rc = lh_get_sizes(h, o);
  if (rc) return rc;
  *s = Sz{o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8], o[9]};
  return LH_OK;
}

// The files of a run with variable-resolution bands keep the middle band's
// planes at its own mode set (per-plane nx, nz records); that layout is not
// written here.
bool banded(const lh_params* prm) {
  return prm->Ngal[1 * 4 + 0] != prm->Ngal[2 * 4 + 0] || prm->Ngal[1 * 4 + 1] != prm->Ngal[2 * 4 + 1];
}

}  // namespace

extern "C" {

int lh_write_restart(lh_handle* h, const lh_params* prm, const double* yu, const double* yv, const char* dir,
                     const char* name, int32_t iter) {
  if (!h || !prm || !dir || !name || !yu || !yv) return LH_EINVAL;
  g_cur = h;
  if (banded(prm)) return io_fail(LH_EUNSUPPORTED, "files of runs with variable-resolution bands are not written");
  Sz s;
  int rc = sizes(h, &s);
  if (rc) return rc;
  const size_t pl = (size_t)s.nkx * s.nz;
  std::vector<double> u1(2 * pl * s.nyu), u2(2 * pl * s.nyv), u3(2 * pl * s.nyu), p(2 * pl * s.nyp);
  if ((rc = lh_get_fields(h, u1.data(), u2.data(), u3.data(), p.data(), LH_LAYOUT_PLANES))) return rc;
  double tm[5];
  if ((rc = lh_get_time(h, tm))) return rc;
  Header hd{};
  hd.t = tm[0];
  hd.Re = prm->Re;
  hd.alp = prm->alp;
  hd.bet = prm->bet;
  hd.mpgx = tm[2];
  hd.nband = 3;
  hd.iter = iter;
  const struct Field { const char* tag; const std::vector<double>* f; int ny, j0; const double* y; } fields[4] = {
      {"u1", &u1, s.nyu, s.ju0, yu}, {"u2", &u2, s.nyv, s.jv0, yv}, {"u3", &u3, s.nyu, s.ju0, yu},
      {"p", &p, s.nyp, s.jp0, yu + 1}};
  for (const Field& fd : fields) {
    const std::string path = std::string(dir) + "/" + fd.tag + name;
    Writer w(path.c_str());
    if (!w.ok) return io_fail(LH_EINVAL, "cannot write " + path);
    w.record(header_parts(hd));
    w.record({{prm->N, 4 * 20}});
    w.record({{fd.y, 8 * (size_t)fd.ny}});
    const int32_t nx = 2 * s.nkx, nz = s.nz;
    for (int jj = 0; jj < fd.ny; ++jj) {
      const int32_t jin = jj + fd.j0, band = 2;
      const double y = fd.y[jj];
      w.record({{&jin, 4}, {&band, 4}, {&nx, 4}, {&nz, 4}, {&y, 8}, {fd.f->data() + 2 * pl * jj, 8 * pl * 2}});
    }
    if (!w.ok) return io_fail(LH_EINVAL, "write failed: " + path);
  }
  return LH_OK;
}

int lh_read_restart(lh_handle* h, const char* dir, const char* name, double* t_out, int32_t* iter_out) {
  if (!h || !dir || !name) return LH_EINVAL;
  g_cur = h;
  Sz s;
  int rc = sizes(h, &s);
  if (rc) return rc;
  const size_t pl = (size_t)s.nkx * s.nz;
  std::vector<double> u1(2 * pl * s.nyu), u2(2 * pl * s.nyv), u3(2 * pl * s.nyu), p(2 * pl * s.nyp);
  const struct Field { const char* tag; std::vector<double>* f; int ny; } fields[4] = {
      {"u1", &u1, s.nyu}, {"u2", &u2, s.nyv}, {"u3", &u3, s.nyu}, {"p", &p, s.nyp}};
  Header hd{};
  std::vector<unsigned char> rec;
  for (const Field& fd : fields) {
    const std::string path = std::string(dir) + "/" + fd.tag + name;
    Reader r(path.c_str());
    if (!r.ok) return io_fail(LH_EINVAL, "cannot open " + path);
    if (r.record(rec) < 48) return io_fail(LH_EINVAL, "bad header in " + path);
    std::memcpy(&hd.t, rec.data(), 8);
    std::memcpy(&hd.nband, rec.data() + 40, 4);
    std::memcpy(&hd.iter, rec.data() + 44, 4);
    if (hd.nband != 3) return io_fail(LH_EINVAL, "wrong startfile? nband in " + path);  // start.f90:1820-1825
    if (r.record(rec) != 80) return io_fail(LH_EINVAL, "bad N record in " + path);
    if (r.record(rec) < 0) return io_fail(LH_EINVAL, "truncated " + path);  // skipped, as read_in does
    for (int jj = 0; jj < fd.ny; ++jj) {
      const long n = r.record(rec);
      if (n < 24) return io_fail(LH_EINVAL, "truncated " + path);
      int32_t nx, nz;
      std::memcpy(&nx, rec.data() + 8, 4);
      std::memcpy(&nz, rec.data() + 12, 4);
      if (nx != 2 * s.nkx || nz != s.nz || (size_t)n != 24 + 8 * (size_t)nx * nz)
        return io_fail(LH_EUNSUPPORTED, "plane size in " + path + " differs from the grid (different N)");
      std::memcpy(fd.f->data() + 2 * pl * jj, rec.data() + 24, 8 * (size_t)nx * nz);
    }
  }
  if ((rc = lh_set_fields(h, u1.data(), u2.data(), u3.data(), p.data(), LH_LAYOUT_PLANES))) return rc;
  if (t_out) *t_out = hd.t;
  if (iter_out) *iter_out = hd.iter;
  return LH_OK;
}

// write_stats (stats.f90:355-410): header, Ngal, (yu, dthetai, dthdyu), (yv, dthetai, dthdyv), istat, the 13
// plane profiles (Um U2m Vm V2m Wm W2m Pm P2m UVm UWm VWm wxm wx2m) and, with canopies, the 13 conditional
// blocks (UmC U2mC VmC V2mC WmC W2mC PmC P2mC UVmC UWmC VWmC wxmC wx2mC), then resets the accumulators as
// write_stats does.
int lh_write_stats(lh_handle* h, const lh_params* prm, const double* yu, const double* yv, const double* dthdyu,
                   const double* dthdyv, const char* path, int32_t iter) {
  if (!h || !prm || !yu || !yv || !dthdyu || !dthdyv || !path) return LH_EINVAL;
  g_cur = h;
  if (banded(prm)) return io_fail(LH_EUNSUPPORTED, "files of runs with variable-resolution bands are not written");
  Sz s;
  int rc = sizes(h, &s);
  if (rc) return rc;
  const int L = s.nyu > s.nyv ? s.nyu : s.nyv;
  std::vector<double> st(13 * (size_t)L);
  int32_t istat = 0, dims[5] = {0, 0, 0, 0, 0}, nc = 0;
  if ((rc = lh_cond_flush(h, nullptr, dims, &nc, 0))) return rc;
  const size_t tile = (size_t)dims[3] * dims[4];
  std::vector<double> cond(tile * (6 * (size_t)dims[0] + 5 * (size_t)dims[1] + 2 * (size_t)dims[2]) + 1);
  if ((rc = lh_cond_flush(h, cond.data(), dims, &nc, 1))) return rc;
  if ((rc = lh_stats_flush(h, st.data(), &istat, 1))) return rc;
  double tm[5];
  if ((rc = lh_get_time(h, tm))) return rc;
  Header hd{};
  hd.t = tm[0]; hd.Re = prm->Re; hd.alp = prm->alp; hd.bet = prm->bet; hd.mpgx = tm[2]; hd.nband = 3; hd.iter = iter;
  const double dthetai = prm->ddthetavi;
  Writer w(path);
  if (!w.ok) return io_fail(LH_EINVAL, std::string("cannot write ") + path);
  w.record(header_parts(hd));
  w.record({{prm->Ngal, 4 * 20}});
  w.record({{yu, 8 * (size_t)s.nyu}, {&dthetai, 8}, {dthdyu, 8 * (size_t)s.nyu}});
  w.record({{yv, 8 * (size_t)s.nyv}, {&dthetai, 8}, {dthdyv, 8 * (size_t)s.nyv}});
  w.record({{&istat, 4}});
  // device rows: 0 Um 1 U2m 2 Vm 3 V2m 4 Wm 5 W2m 6 Pm 7 P2m 8 UVm 9 UWm 10 VWm 11 wxm 12 wx2m, written in that
  // order (recvX, stats.f90:369-382)
  const int ny_of[13] = {s.nyu, s.nyu, s.nyv, s.nyv, s.nyu, s.nyu, s.nyp, s.nyp, s.nyu, s.nyu, s.nyv, s.nyv, s.nyv};
  for (int r = 0; r < 13; ++r) w.record({{st.data() + (size_t)r * L, 8 * (size_t)ny_of[r]}});
  if (tile) {
    // device block order: UmC U2mC WmC W2mC UVmC UWmC | VmC V2mC VWmC | PmC P2mC | wxmC wx2mC
    const size_t bu = tile * dims[0], bv = tile * dims[1], bp = tile * dims[2];
    const double* c = cond.data();
    const double *UmC = c, *U2mC = c + bu, *WmC = c + 2 * bu, *W2mC = c + 3 * bu, *UVmC = c + 4 * bu, *UWmC = c + 5 * bu;
    const double *VmC = c + 6 * bu, *V2mC = VmC + bv, *VWmC = VmC + 2 * bv;
    const double *PmC = VmC + 3 * bv, *P2mC = PmC + bp;
    const double *wxmC = P2mC + bp, *wx2mC = wxmC + bv;
    const std::pair<const double*, size_t> recs[13] = {{UmC, bu}, {U2mC, bu}, {VmC, bv}, {V2mC, bv}, {WmC, bu},
                                                       {W2mC, bu}, {PmC, bp}, {P2mC, bp}, {UVmC, bu}, {UWmC, bu},
                                                       {VWmC, bv}, {wxmC, bv}, {wx2mC, bv}};
    for (const auto& rr : recs) w.record({{rr.first, 8 * rr.second}});
  }
  if (!w.ok) return io_fail(LH_EINVAL, std::string("write failed: ") + path);
  return LH_OK;
}

// recvwrspec (spectra.f90:109-180), one file per quantity <dir>/<spU_|spV_|spW_|spUV_|spP_><name>: header, N,
// (yu, dthetai, dthdyu), (yv, dthetai, dthdyv), the count, and buffSP(0:N1/2, 1:N2/2+1, j) with kz and -kz
// folded into one slot (the +1 slot holds kz = -N2/2) and the kx >= 1 columns doubled.  The reference assigns
// rank 0's own columns and adds the others' (so with one rank the -kz sums overwrite the +kz ones); here the
// two are added, which is what the fold is for.  Resets the accumulators.
int lh_write_spectra(lh_handle* h, const lh_params* prm, const double* yu, const double* yv, const double* dthdyu,
                     const double* dthdyv, const char* dir, const char* name, int32_t iter) {
  if (!h || !prm || !yu || !yv || !dthdyu || !dthdyv || !dir || !name) return LH_EINVAL;
  g_cur = h;
  if (banded(prm)) return io_fail(LH_EUNSUPPORTED, "files of runs with variable-resolution bands are not written");
  Sz s;
  int rc = sizes(h, &s);
  if (rc) return rc;
  const size_t np = (size_t)s.nkx * s.nz;
  std::vector<double> spU(np * s.nyu), spV(np * s.nyv), spW(np * s.nyu), spUV(np * s.nyu), spP(np * s.nyp);
  int32_t count = 0;
  if ((rc = lh_spectra_flush(h, spU.data(), spV.data(), spW.data(), spUV.data(), spP.data(), &count, 1))) return rc;
  double tm[5];
  if ((rc = lh_get_time(h, tm))) return rc;
  Header hd{};
  hd.t = tm[0]; hd.Re = prm->Re; hd.alp = prm->alp; hd.bet = prm->bet; hd.mpgx = tm[2]; hd.nband = 3; hd.iter = iter;
  const double dthetai = prm->ddthetavi;
  const int nkx = s.nkx, nz = s.nz, nh = nz / 2 + 1;
  const struct Q { const char* tag; const std::vector<double>* v; int ny; } qs[5] = {
      {"spU_", &spU, s.nyu}, {"spV_", &spV, s.nyv}, {"spW_", &spW, s.nyu}, {"spUV_", &spUV, s.nyu}, {"spP_", &spP, s.nyp}};
  for (const Q& q : qs) {
    std::vector<double> buf((size_t)nkx * nh * q.ny, 0.0);
    for (int j = 0; j < q.ny; ++j)
      for (int kk = 0; kk < nz; ++kk) {
        const int k = kk + 1;                           // reference column index k
        const int kf = (k > nz / 2) ? nz + 2 - k : k;   // folded slot, 1-based
        for (int i = 0; i < nkx; ++i)
          buf[((size_t)j * nh + (kf - 1)) * nkx + i] += (*q.v)[(size_t)j * np + (size_t)kk * nkx + i];
      }
    for (int j = 0; j < q.ny; ++j)
      for (int k = 0; k < nh; ++k)
        for (int i = 1; i < nkx; ++i) buf[((size_t)j * nh + k) * nkx + i] *= 2.0;
    const std::string path = std::string(dir) + "/" + q.tag + name;
    Writer w(path.c_str());
    if (!w.ok) return io_fail(LH_EINVAL, "cannot write " + path);
    w.record(header_parts(hd));
    w.record({{prm->N, 4 * 20}});
    w.record({{yu, 8 * (size_t)s.nyu}, {&dthetai, 8}, {dthdyu, 8 * (size_t)s.nyu}});
    w.record({{yv, 8 * (size_t)s.nyv}, {&dthetai, 8}, {dthdyv, 8 * (size_t)s.nyv}});
    w.record({{&count, 4}});
    w.record({{buf.data(), 8 * buf.size()}});
    if (!w.ok) return io_fail(LH_EINVAL, "write failed: " + path);
  }
  return LH_OK;
}

}  // extern "C"
