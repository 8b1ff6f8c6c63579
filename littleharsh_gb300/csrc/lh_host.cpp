// lh_host.cpp -- host-side setup for drivers without a Fortran compiler.
//
// Restates the parts of the reference's start-up that produce what lh_init
// consumes: the input.in reader (start.f90:63-196 with the FORMATs of
// start.f90:433-436), the stretched y grid (y_grid_canopy.f90:24-194), the
// ghost-point weights (start.f90:497-503) and the canopy point lists
// (geom_sym_canopy.f90:63-234).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/littleharsh.h"

namespace {

// x**n for integer n, evaluated the way Fortran does (repeated squaring).
double ipow(double x, int n) {
  unsigned e = (unsigned)(n < 0 ? -n : n);
  double r = (e & 1u) ? x : 1.0;
  while ((e >>= 1) != 0) {
    x *= x;
    if (e & 1u) r *= x;
  }
  return n < 0 ? 1.0 / r : r;
}

// Characters [skip, skip+width) of a record, blank padded.
std::string column(const std::string& rec, size_t skip, size_t width) {
  std::string out(width, ' ');
  for (size_t c = 0; c < width && skip + c < rec.size(); ++c) out[c] = rec[skip + c];
  return out;
}

std::string squeeze(const std::string& f) {
  std::string s;
  for (char c : f)
    if (c != ' ' && c != '\t' && c != '\r' && c != '\n') s += c;
  return s;
}

// Iw edit descriptor on input.
bool read_I(const std::string& f, int32_t* v) {
  std::string s = squeeze(f);
  if (s.empty()) { *v = 0; return true; }
  char* end = nullptr;
  long x = std::strtol(s.c_str(), &end, 10);
  if (*end) return false;
  *v = (int32_t)x;
  return true;
}

// Dw.1 edit descriptor on input: optional exponent letter (D, E, Q) or a bare
// signed exponent; a mantissa without '.' carries one implied decimal.
bool read_D(const std::string& f, double* v) {
  std::string s = squeeze(f);
  if (s.empty()) { *v = 0.0; return true; }
  size_t ep = std::string::npos;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = (char)std::toupper((unsigned char)s[i]);
    if (c == 'D' || c == 'E' || c == 'Q') { ep = i; break; }
    if ((c == '+' || c == '-') && i > 0) { ep = i; break; }
  }
  std::string mant = s.substr(0, ep == std::string::npos ? s.size() : ep);
  long ex = 0;
  if (ep != std::string::npos) {
    std::string es = s.substr(std::isalpha((unsigned char)s[ep]) ? ep + 1 : ep);
    char* end = nullptr;
    ex = std::strtol(es.c_str(), &end, 10);
    if (*end) return false;
  }
  if (mant.find('.') == std::string::npos) ex -= 1;
  char* end = nullptr;
  std::strtod(mant.c_str(), &end);
  if (*end || mant.empty()) return false;
  std::string full = mant + "e" + std::to_string(ex);
  *v = std::strtod(full.c_str(), nullptr);
  return true;
}

void read_A(const std::string& f, char* out, size_t n) {
  size_t len = f.size();
  while (len > 0 && f[len - 1] == ' ') --len;
  if (len >= n) len = n - 1;
  std::memcpy(out, f.data(), len);
  out[len] = 0;
}

}  // namespace

extern "C" int lh_read_input(const char* path, lh_input* in) {
  if (!path || !in) return LH_EINVAL;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return LH_EINVAL;
  std::vector<std::string> rec;
  char buf[1024];
  while (std::fgets(buf, sizeof buf, fp)) {
    std::string s(buf);
    while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
    rec.push_back(s);
  }
  std::fclose(fp);
  std::memset(in, 0, sizeof *in);
  size_t r = 0;
  bool ok = true;
  auto next = [&]() -> const std::string* {
    if (r >= rec.size()) { ok = false; return nullptr; }
    return &rec[r++];
  };
  auto skip = [&](int n) { for (int i = 0; i < n; ++i) next(); };
  auto D = [&](double* v) { const std::string* s = next(); if (s && !read_D(column(*s, 7, 10), v)) ok = false; };
  auto I = [&](int32_t* v) { const std::string* s = next(); if (s && !read_I(column(*s, 7, 10), v)) ok = false; };
  auto A = [&](char* v, size_t n) { const std::string* s = next(); if (s) read_A(column(*s, 7, 90), v, n); };
  skip(9);
  D(&in->Re); skip(2);
  D(&in->alp); D(&in->bet);
  I(&in->ngalx1); I(&in->ngalx2); I(&in->ngalz1); I(&in->ngalz2); I(&in->ny);
  D(&in->dyq); I(&in->ppp); skip(2);
  I(&in->flag_init); skip(3);
  A(in->fnameimb, sizeof in->fnameimb); skip(1);
  A(in->dirin, sizeof in->dirin); A(in->dirout, sizeof in->dirout); skip(2);
  D(&in->CFL); I(&in->nwrite);
  {
    const std::string* s = next();
    if (s && !read_I(column(*s, 12, 5), &in->flag_ctpress)) ok = false;
  }
  skip(1);
  if (!ok) return LH_EINVAL;
  if (in->flag_ctpress == 1) D(&in->mpgx);
  else if (in->flag_ctpress == 0) skip(1);
  else return LH_EINVAL;  // "Wrong presure flag"
  skip(3);
  D(&in->Kib); D(&in->maxerr); D(&in->maxt); D(&in->maxA);
  in->maxA = -in->maxA;
  I(&in->physlim_bot); I(&in->physlim_top); skip(2);
  I(&in->geometry_type); skip(4);
  I(&in->ntilex); I(&in->ntilez);
  if (ok && in->geometry_type != 0 && (in->ntilex <= 0 || in->ntilez <= 0)) return LH_EINVAL;  // "Tiles must be positive"
  D(&in->posth); I(&in->npeakx); I(&in->npeakz); D(&in->Lfracx); D(&in->Lfracz);
  I(&in->dsty); I(&in->dstx); I(&in->dstz);
  if (!ok) return LH_EINVAL;
  if (in->geometry_type == 2 && (in->npeakx <= 0 || in->npeakz <= 0)) return LH_EINVAL;
  if (in->geometry_type == 3 && (in->dstx <= 0 || in->dstz <= 0 || in->dsty <= 0)) return LH_EINVAL;
  return LH_OK;
}

extern "C" int lh_setup_grid(const lh_input* in, lh_params* prm, double* yu_o, double* yv_o, double* dthdyu_o,
                             double* dthdyv_o, double* dyu2i_o, double* dyv2i_o) {
  if (!in || !prm) return LH_EINVAL;
  if (in->ny < 8 || in->ppp < 3 || in->dsty < 0) return LH_EINVAL;
  // h_ny(1) and the effective canopy height (start.f90:214-240)
  double posth = in->posth, hny;
  switch (in->geometry_type) {
    case 0: posth = 0.0; hny = 0.25; break;
    case 3: hny = 1.5 * posth; break;
    default: return LH_EUNSUPPORTED;  // only canopies (and no canopy) have a forcing builder
  }
  const int dny = in->dsty;
  const int nnt = in->ny - 1;  // points between the tips minus one: nn inside y_grid_canopy
  const int jlo = -dny;
  const int nyu = nnt + 2 * dny + 2, nyv = nnt + 2 * dny + 1;
  std::vector<double> yu(nyu), yv(nyv), tu(nyu), tv(nyv), du(3 * nyu), dv(3 * nyv);
  auto YU = [&](int j) -> double& { return yu[j - jlo]; };
  auto YV = [&](int j) -> double& { return yv[j - jlo]; };
  auto TU = [&](int j) -> double& { return tu[j - jlo]; };
  auto TV = [&](int j) -> double& { return tv[j - jlo]; };
  const int p = in->ppp;
  const double dyq = in->dyq, q = nnt / 2.0;
  const double den = 8.0 * dyq + 7.0;
  const double A = 15.0 * (dyq - 1.0) / (den * ipow(q, p));
  const double B = -30.0 * (dyq - 1.0) / (den * ipow(q, p - 2));
  const double Cc = 15.0 * dyq / (den * q);
  auto ymap = [&](double s) { return A * ipow(s, p) / 5.0 + B * ipow(s, p - 2) / 3.0 + Cc * s; };
  auto dmap = [&](double s) { return 1.0 / (A * ipow(s, p - 1) + B * ipow(s, p - 3) + Cc); };
  for (int j = 0; j < nnt; ++j) {
    YV(j) = ymap(j - q);
    YU(j + 1) = ymap(j + 0.5 - q);
    TV(j) = dmap(j - q);
    TU(j + 1) = dmap(j + 0.5 - q);
  }
  if (dny == 0) {
    YU(0) = ymap(-0.5 - q);
    TU(0) = dmap(-0.5 - q);
    // top wall and its ghost: left unset by the reference for dsty = 0
    YV(nnt) = ymap(nnt - q);
    TV(nnt) = dmap(nnt - q);
    YU(nnt + 1) = ymap(nnt + 0.5 - q);
    TU(nnt + 1) = dmap(nnt + 0.5 - q);
  } else {
    const double g = YV(1) - YV(0);
    const double a1 = -(15.0 * (posth - g * dny)) / (7.0 * std::pow((double)dny, 5.0));
    const double c1 = (30.0 * (posth - g * dny)) / (7.0 * std::pow((double)dny, 3.0));
    auto cmap_half = [&](double s) { return a1 * ipow(s, 5) / 5.0 + c1 * ipow(s, 3) / 3.0 + g * s; };
    auto cder_half = [&](double s) { return 1.0 / (a1 * ipow(s, 4) + c1 * ipow(s, 2) + g); };
    auto cmap_int = [&](int j) {
      const double s = (double)j;
      return a1 * std::pow(s, 5.0) / 5.0 + c1 * std::pow(s, 3.0) / 3.0 + g * s;
    };
    auto cder_int = [&](int j) { return 1.0 / (a1 * (double)(j * j * j * j) + c1 * (double)(j * j) + g); };
    YU(-dny) = cmap_half(-dny - 0.5) - 1.0;
    TU(-dny) = cder_half(-dny - 0.5);
    for (int j = -dny; j <= -1; ++j) {
      YV(j) = cmap_int(j) - 1.0;
      YU(j + 1) = cmap_half(j + 0.5) - 1.0;
      TV(j) = cder_int(j);
      TU(j + 1) = cder_half(j + 0.5);
    }
    for (int j = 0; j <= dny; ++j) {
      YV(j + nnt) = cmap_int(j) + 1.0;
      YU(j + nnt + 1) = cmap_half(j + 0.5) + 1.0;
      TV(j + nnt) = cder_int(j);
      TU(j + nnt + 1) = cder_half(j + 0.5);
    }
  }
  // second-derivative stencils
  auto D2 = [&](std::vector<double>& c, int idx0, const std::vector<double>& y, int j, int kind) {
    const double ym = kind == 1 ? 0 : y[j - jlo - 1], y0 = y[j - jlo], yp = kind == 2 ? 0 : y[j - jlo + 1];
    double* o = &c[3 * (j - idx0)];
    if (kind == 0) {
      o[0] = 2.0 / ((y0 - ym) * (yp - ym));
      o[1] = -2.0 / ((yp - y0) * (y0 - ym));
      o[2] = 2.0 / ((yp - y0) * (yp - ym));
    } else if (kind == 1) {  // first point: one-sided
      o[0] = 0.0;
      o[1] = -2.0 / ipow(yp - y0, 2);
      o[2] = 1.0 / ipow(yp - y0, 2);
    } else {  // last point
      o[0] = 1.0 / ipow(y0 - ym, 2);
      o[1] = -2.0 / ipow(y0 - ym, 2);
      o[2] = 0.0;
    }
  };
  D2(du, jlo, yu, jlo, 1);
  D2(dv, jlo, yv, jlo, 1);
  for (int j = jlo + 1; j <= nnt + dny - 1; ++j) { D2(du, jlo, yu, j, 0); D2(dv, jlo, yv, j, 0); }
  D2(du, jlo, yu, nnt + dny, 0);
  D2(dv, jlo, yv, nnt + dny, 2);
  D2(du, jlo, yu, nnt + dny + 1, 2);
  // band bookkeeping (y_grid_canopy.f90:147-187)
  int N[4][5] = {{0}}, G[4][5] = {{0}};
  G[0][1] = in->ngalx1; G[0][2] = in->ngalx2; G[0][3] = in->ngalx1; G[0][4] = -2;
  G[1][1] = in->ngalz1; G[1][2] = in->ngalz2; G[1][3] = in->ngalz1; G[1][4] = 0;
  G[2][3] = in->ny - 2;
  std::memcpy(N, G, sizeof N);
  for (int b = 1; b <= 3; ++b) { N[0][b] = 2 * (G[0][b] / 3); N[1][b] = 2 * (G[1][b] / 3); }
  const int nn = in->ny - 2;
  N[2][0] = -dny; N[3][0] = -dny;
  {
    int j = -dny;
    const double h = YU(0) + hny;
    while (j - jlo < nyu && YU(j) < h) ++j;
    N[2][1] = j;
    N[2][2] = N[2][3] - j;
  }
  N[2][3] = nn + dny;
  N[3][1] = N[2][1] + 1;
  N[3][2] = N[2][2];
  N[3][3] = N[2][3] + 1;
  for (int b = 0; b <= 4; ++b) { G[2][b] = N[2][b]; G[3][b] = N[3][b]; }
  // ghost-point weights (start.f90:497-503), indices relative to the grids
  const int n30 = N[2][0], n40 = N[3][0], n31 = N[2][1], n41 = N[3][1], n32 = N[2][2], n42 = N[3][2],
            n33 = N[2][3], n43 = N[3][3];
  double gw[3][2];
  gw[0][0] = -(YV(n30) - YU(n40)) / (YV(n30) - YU(n40 + 1));
  gw[0][1] = (YU(n41 + 1) - YV(n31 + 1)) / (YV(n31 + 1) - YU(n41));
  gw[1][0] = -(YV(n30) - YU(n40)) / (YV(n30) - YU(n40 + 1));
  gw[1][1] = (YU(n43 + 1) - YV(n33 + 1)) / (YV(n33 + 1) - YU(n43));
  gw[2][0] = -(YV(n32) - YU(n42)) / (YV(n32) - YU(n42 + 1));
  gw[2][1] = (YU(n43 + 1) - YV(n33 + 1)) / (YV(n33 + 1) - YU(n43));
  // fill the parameter block
  prm->abi_version = LH_ABI_VERSION;
  for (int b = 0; b <= 4; ++b)
    for (int r = 0; r < 4; ++r) { prm->N[b * 4 + r] = N[r][b]; prm->Ngal[b * 4 + r] = G[r][b]; }
  prm->nn = nn;
  prm->flag_ctpress = in->flag_ctpress;
  prm->geometry_type = in->geometry_type;
  prm->dsty = in->dsty;
  prm->Re = in->Re; prm->alp = in->alp; prm->bet = in->bet;
  prm->ddthetavi = 1.0;
  prm->ntilex = in->ntilex;
  prm->ntilez = in->ntilez;
  for (int c = 0; c < 2; ++c)
    for (int b = 0; b < 3; ++b) prm->gridweighting[c * 3 + b] = gw[b][c];
  if (yu_o) std::memcpy(yu_o, yu.data(), sizeof(double) * nyu);
  if (yv_o) std::memcpy(yv_o, yv.data(), sizeof(double) * nyv);
  if (dthdyu_o) std::memcpy(dthdyu_o, tu.data(), sizeof(double) * nyu);
  if (dthdyv_o) std::memcpy(dthdyv_o, tv.data(), sizeof(double) * nyv);
  if (dyu2i_o) std::memcpy(dyu2i_o, du.data(), sizeof(double) * 3 * nyu);
  if (dyv2i_o) std::memcpy(dyv2i_o, dv.data(), sizeof(double) * 3 * nyv);
  return LH_OK;
}

extern "C" int lh_setup_canopy(const lh_input* in, const lh_params* prm, int32_t* list_u, int32_t* nlist_u,
                               int32_t* list_v, int32_t* nlist_v) {
  if (!in || !prm || !nlist_u || !nlist_v) return LH_EINVAL;
  if (in->geometry_type != 3) { *nlist_u = 0; *nlist_v = 0; return LH_OK; }
  const int ngx = prm->Ngal[1 * 4 + 0], ngz = prm->Ngal[1 * 4 + 1];
  if (in->ntilex == 0 || in->ntilez == 0) return LH_EINVAL;
  // the reference tests Ngal(1,1) and Ngal(2,1) against ntilez (geom_sym_canopy.f90:54,58)
  if (ngx % in->ntilez != 0 || ngz % in->ntilez != 0) return LH_EINVAL;
  const int dnx = ngx / in->ntilex, dnz = ngz / in->ntilez, dsty = in->dsty;
  const int ngal43 = prm->Ngal[3 * 4 + 3], ngal33 = prm->Ngal[3 * 4 + 2];
  const int stem = dsty * in->dstx * in->dstz;
  const int per = in->ntilex * in->ntilez * stem;  // points per canopy and grid
  if (!list_u || !list_v) { *nlist_u = 2 * per; *nlist_v = 2 * per; return LH_OK; }
  if (*nlist_u < 2 * per || *nlist_v < 2 * per) return LH_EINVAL;
  // j ranges of the stems: lower canopy, then upper (the upper v list is shifted by -1)
  const int ju[2][2] = {{-dsty + 1, 0}, {ngal43 - dsty + 1, ngal43}};
  const int jv[2][2] = {{-dsty, -1}, {ngal33 + 1 - dsty + 1, ngal33 + 1}};
  int nu = 0, nv = 0;
  for (int c = 0; c < 2; ++c) {
    for (int grid = 0; grid < 2; ++grid) {
      int32_t* L = grid == 0 ? list_u : list_v;
      int& n = grid == 0 ? nu : nv;
      const int ja = grid == 0 ? ju[c][0] : jv[c][0], jb = grid == 0 ? ju[c][1] : jv[c][1];
      const int shift = (grid == 1 && c == 1) ? -1 : 0;
      // one stem, then its copies tile by tile (x tiles outer, z tiles inner)
      for (int ix = 1; ix <= in->ntilex; ++ix)
        for (int iz = 1; iz <= in->ntilez; ++iz)
          for (int j = ja; j <= jb; ++j)
            for (int i = 1; i <= in->dstx; ++i)
              for (int k = 1; k <= in->dstz; ++k) {
                L[3 * n + 0] = i + dnx * (ix - 1);
                L[3 * n + 1] = k + dnz * (iz - 1);
                L[3 * n + 2] = j + shift;
                ++n;
              }
    }
  }
  *nlist_u = nu;
  *nlist_v = nv;
  return LH_OK;
}
