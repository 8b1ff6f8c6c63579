// lh_noalloc.cu -- divergence-free projection for callers that cannot allocate
// device memory.
//
// Some callers own every byte of device memory themselves: a Fortran driver
// whose fields live in OpenACC or CUDA Fortran device arrays, or an
// application that carves all GPU memory out of one arena at start-up and
// must not call cudaMalloc later (an allocation in the middle of a run can
// synchronise the device and breaks a fixed memory budget).  Such a caller
// cannot create an lh_handle, because lh_init allocates the solver's fields
// and tables.  lh_project_noalloc gives it the projection step on its own
// device arrays: the caller passes the velocity fields, and every scratch
// buffer (wavenumbers, metric, the per-column pressure LU, psi, p) lives in
// the file-scope array below.  Nothing here calls cudaMalloc, cudaFree or an
// allocating library routine.
//
// The array is kNoAllocScratchBytes (64 MiB) on every GPU that loads this
// library, held until the process exits.  It is shared by all calls, keeps
// the contents of the last call, and calls whose work overlaps on the GPU
// race on it.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/littleharsh.h"
#include "lh_internal.h"

using namespace lh;

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Failures are reported through lh_last_error(NULL).
int na_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_init_error(buf);
  return code;
}

// Device address of the scratch array on the current device.  The name of a
// __device__ array is only a host-side stand-in, so the address is looked up
// with that device current, on every call: a cached address would go stale
// after cudaDeviceReset, which unloads the module.  The lookup is cheap next
// to the solve.
int scratch_address(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return na_fail(LH_ECUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  *out = static_cast<unsigned char*>(p);
  return LH_OK;
}

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" int lh_project_noalloc(const lh_params* prm, const double* yu, const double* dthdyu,
                                  const double* dthdyv, double* u1, double* u2, double* u3, double dt,
                                  void* stream) {
  if (!prm || !yu || !dthdyu || !dthdyv || !u1 || !u2 || !u3) return na_fail(LH_EINVAL, "NULL argument");
  if (prm->abi_version != LH_ABI_VERSION) return na_fail(LH_EINVAL, "abi_version %d", prm->abi_version);
  if (!(dt > 0.0)) return na_fail(LH_EINVAL, "dt must be positive");
  // the checks lh_init makes on the parameter block
  Dims d{};
  {
    std::string why;
    const int rc = make_dims(prm, &d, &why);
    if (rc) return na_fail(rc, "%s", why.c_str());
  }
  if (d.banded) return na_fail(LH_EUNSUPPORTED, "bands with different x/z resolutions are not built");
  const int nz = d.nz;
  // scratch layout
  const size_t np = (size_t)d.np, nyp = (size_t)d.nyp;
  const size_t o_kx = 0, o_kz = o_kx + up256(8 * (size_t)d.nkx), o_k2x = o_kz + up256(8 * (size_t)nz),
               o_k2z = o_k2x + up256(8 * (size_t)d.nkx), o_cu = o_k2z + up256(8 * (size_t)nz),
               o_cv = o_cu + up256(8 * (size_t)d.nyu), o_rows = o_cv + up256(8 * (size_t)d.nyv),
               o_dg1 = o_rows + up256(32 * nyp), o_dg2 = o_dg1 + up256(8 * nyp),
               o_dg3 = o_dg2 + up256(8 * nyp * np), o_psi = o_dg3 + up256(8 * nyp * np),
               o_p = o_psi + up256(16 * nyp * np), total = o_p + up256(16 * nyp * np);
  if (total > kNoAllocScratchBytes)
    return na_fail(LH_EINVAL, "grid needs %zu bytes of scratch; lh_project_noalloc is limited to %zu bytes", total,
                   kNoAllocScratchBytes);
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  // host tables (the same formulas as lh_init)
  const double alp = prm->alp, bet = prm->bet, dv = prm->ddthetavi;
  std::vector<double> kx(d.nkx), k2x(d.nkx), kz(nz), k2z(nz), cu(d.nyu), cv(d.nyv), rows(4 * nyp), dg1(nyp);
  for (int i = 0; i < d.nkx; ++i) { kx[i] = alp * i; k2x[i] = -((alp * i) * (alp * i)); }
  for (int k = 1; k <= nz; ++k) {
    const double a = k <= nz / 2 ? bet * (k - 1) : bet * (nz - k + 1);
    kz[k - 1] = k <= nz / 2 ? a : -a;
    k2z[k - 1] = -(a * a);
  }
  for (int j = 0; j < d.nyu; ++j) cu[j] = dv * dthdyu[j];
  for (int j = 0; j < d.nyv; ++j) cv[j] = dv * dthdyv[j];
  for (size_t jp = 0; jp < nyp; ++jp) {
    const size_t ju = jp + 1, jf = jp + 1;
    const double Dt = dv * dthdyu[ju], Dbm = -dv * dthdyu[ju];
    const double Gb = -dv * dthdyv[jf], Gtp = dv * dthdyv[jf];
    const double Gt = jp > 0 ? dv * dthdyv[jf - 1] : 0.0, Gbm = jp > 0 ? -dv * dthdyv[jf - 1] : 0.0;
    rows[4 * jp + 0] = Dbm * Gt;
    rows[4 * jp + 1] = Dt * Gb;
    rows[4 * jp + 2] = Dbm * Gbm;
    rows[4 * jp + 3] = Dt * Gtp;
    dg1[jp] = rows[4 * jp + 2];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  struct Up { size_t off; const std::vector<double>* v; } ups[] = {
      {o_kx, &kx}, {o_kz, &kz}, {o_k2x, &k2x}, {o_k2z, &k2z}, {o_cu, &cu}, {o_cv, &cv}, {o_rows, &rows}, {o_dg1, &dg1}};
  for (const Up& u : ups) {
    cudaError_t e = cudaMemcpyAsync(base + u.off, u.v->data(), u.v->size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return na_fail(LH_ECUDA, "table upload: %s", cudaGetErrorString(e));
  }
  Tables t{};
  t.kx = reinterpret_cast<const double*>(base + o_kx);
  t.kz = reinterpret_cast<const double*>(base + o_kz);
  t.k2x = reinterpret_cast<const double*>(base + o_k2x);
  t.k2z = reinterpret_cast<const double*>(base + o_k2z);
  t.cu = reinterpret_cast<const double*>(base + o_cu);
  t.cv = reinterpret_cast<const double*>(base + o_cv);
  t.dg1 = reinterpret_cast<const double*>(base + o_dg1);
  double* dg2 = reinterpret_cast<double*>(base + o_dg2);
  double* dg3 = reinterpret_cast<double*>(base + o_dg3);
  t.dg2 = dg2;
  t.dg3 = dg3;
  double2* psi = reinterpret_cast<double2*>(base + o_psi);
  double2* p = reinterpret_cast<double2*>(base + o_p);
  const double dy12 = yu[2 - d.ju0] - yu[1 - d.ju0];
  launch_build_dg(dg2, dg3, reinterpret_cast<const double*>(base + o_rows), d, t, 1.0 / (dy12 * dy12), st);
  // p is accumulated into (p += psi): it must start at zero on every call
  cudaError_t e = cudaMemsetAsync(p, 0, 16 * nyp * np, st);
  if (e != cudaSuccess) return na_fail(LH_ECUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
  const double ab = 4.0 / 15.0 + 4.0 / 15.0;  // aRK(1) + bRK(1)
  const double dtirk = (1.0 / dt) / ab, dtrk = dt * ab;
  const double gwb = prm->gridweighting[0], gwt = prm->gridweighting[3 + 2];  // gridweighting(1,1), (3,2)
  launch_psolve(reinterpret_cast<double2*>(u1), reinterpret_cast<double2*>(u2), reinterpret_cast<double2*>(u3), p,
                psi, d, t, dtirk, dtrk, gwb, gwt, nullptr, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(LH_ECUDA, "launch: %s", cudaGetErrorString(e));
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return na_fail(LH_ECUDA, "projection: %s", cudaGetErrorString(e));
  return LH_OK;
}
