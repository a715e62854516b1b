// tlr_points.cu -- pointwise entry points for the golden tests:
// LNSCoefficients::evaluate on arbitrary base-flow points (including the x
// derivatives that the BiGlobal assembly sets to zero) and the Fourier and
// curvilinear transforms on arbitrary physical blocks.  Compiled with
// --fmad=false like the assembly.
#include <cfloat>

#include "tlr_internal.h"
#include "tlr_lns.cuh"

namespace tlr {
namespace {

__device__ inline bool finite(double v) { return isfinite(v); }

struct PointParams {
  int np;
  double Re, Pr, M, gamma, s;
};

struct LnsBody {
  const FlowPoint &f;
  const Transport &tr;
  double *o;
  bool &ok;
  template <int RC>
  __device__ __forceinline__ void operator()() {
    const Entry e = phys_entry<RC>(f, tr);
    const double vals[11] = {e.G, e.A, e.B, e.C, e.D, e.Vxx,
                             e.Vxy, e.Vxz, e.Vyy, e.Vyz, e.Vzz};
    for (int b = 0; b < 11; ++b) {
      o[b * 25 + RC] = vals[b];
      ok = ok && finite(vals[b]);
    }
  }
};

__global__ void k_lns_points(PointParams p, const double *__restrict__ q,
                             double *__restrict__ out, int *status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.np) return;
  const double *v = q + (size_t)t * 50;
  for (int k = 0; k < 50; ++k)
    if (!finite(v[k])) { status[t] = 1; return; }
  FlowPoint f;
  f.rho = v[0]; f.U = v[1]; f.V = v[2]; f.W = v[3]; f.T = v[4];
  f.rhox = v[5]; f.Ux = v[6]; f.Vx = v[7]; f.Wx = v[8]; f.Tx = v[9];
  f.rhoy = v[10]; f.Uy = v[11]; f.Vy = v[12]; f.Wy = v[13]; f.Ty = v[14];
  f.rhoz = v[15]; f.Uz = v[16]; f.Vz = v[17]; f.Wz = v[18]; f.Tz = v[19];
  f.Uxx = v[21]; f.Vxx = v[22]; f.Wxx = v[23]; f.Txx = v[24];
  f.Uyy = v[26]; f.Vyy = v[27]; f.Wyy = v[28]; f.Tyy = v[29];
  f.Uzz = v[31]; f.Vzz = v[32]; f.Wzz = v[33]; f.Tzz = v[34];
  f.Uxy = v[36]; f.Vxy = v[37]; f.Wxy = v[38];
  f.Uxz = v[41]; f.Vxz = v[42]; f.Wxz = v[43];
  f.Uyz = v[46]; f.Vyz = v[47]; f.Wyz = v[48];
  if (f.rho <= 0.0) { status[t] = 2; return; }
  if (f.T <= 0.0) { status[t] = 3; return; }
  const Transport tr = transport(f, p.Re, p.Pr, p.M, p.gamma, p.s);
  double *o = out + (size_t)t * 275;
  bool ok = true;
  LnsBody body{f, tr, o, ok};
  for_entries<0>(body);
  status[t] = ok ? 0 : 4;
}

__global__ void k_transform_points(int np, const double *__restrict__ alpha,
                                   const double *__restrict__ phys,
                                   const double *__restrict__ met,
                                   double *__restrict__ four,
                                   double *__restrict__ curv, int *status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const double ar = alpha[2 * t], ai = alpha[2 * t + 1];
  const double *ph = phys + (size_t)t * 275;
  const double *mm = met + (size_t)t * 10;
  bool ok = finite(ar) && finite(ai);
  for (int k = 0; k < 275; ++k) ok = ok && finite(ph[k]);
  for (int k = 0; k < 10; ++k) ok = ok && finite(mm[k]);
  if (!ok) { status[t] = 1; return; }
  const double ia_re = 0.0 * ar - 1.0 * ai, ia_im = 0.0 * ai + 1.0 * ar;
  const double a2_re = ar * ar - ai * ai, a2_im = ar * ai + ai * ar;
  Metric10 m{mm[0], mm[1], mm[2], mm[3], mm[4], mm[5], mm[6], mm[7], mm[8], mm[9]};
  double *fo = four + (size_t)t * 350, *co = curv + (size_t)t * 350;
  bool fin = true;
  for (int rc = 0; rc < 25; ++rc) {
    Entry e;
    e.G = ph[rc]; e.A = ph[25 + rc]; e.B = ph[50 + rc]; e.C = ph[75 + rc];
    e.D = ph[100 + rc]; e.Vxx = ph[125 + rc]; e.Vxy = ph[150 + rc];
    e.Vxz = ph[175 + rc]; e.Vyy = ph[200 + rc]; e.Vyz = ph[225 + rc];
    e.Vzz = ph[250 + rc];
    const FourierEntry f = fourier_entry_full(e, ia_re, ia_im, a2_re, a2_im);
    const CurvEntry c = curv_entry_full(f, m);
    const double fv[14] = {f.G, 0.0, f.K0r, f.K0i, f.Kyr, f.Kyi, f.Kzr, f.Kzi,
                           f.Vyy, 0.0, f.Vyz, 0.0, f.Vzz, 0.0};
    const double cv[14] = {c.G, 0.0, c.K0r, c.K0i, c.Kxr, c.Kxi, c.Ker, c.Kei,
                           c.Vxx, 0.0, c.Vxe, 0.0, c.Vee, 0.0};
    for (int b = 0; b < 7; ++b) {
      fo[b * 50 + 2 * rc] = fv[2 * b];
      fo[b * 50 + 2 * rc + 1] = fv[2 * b + 1];
      co[b * 50 + 2 * rc] = cv[2 * b];
      co[b * 50 + 2 * rc + 1] = cv[2 * b + 1];
    }
    for (int k = 0; k < 14; ++k) fin = fin && finite(fv[k]) && finite(cv[k]);
  }
  status[t] = fin ? 0 : 4;
}

template <typename T>
cudaError_t up(T **d, const T *h, size_t n) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(d), n * sizeof(T));
  if (e != cudaSuccess) return e;
  return h ? cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) : cudaSuccess;
}

}  // namespace
}  // namespace tlr

using namespace tlr;

extern "C" int tlr_lns_points(const tlr_recipe *r, int np, const double *q,
                              double *blocks, int *status) {
  if (!r || np <= 0 || !q || !blocks || !status) return TLR_ERR_ARG;
  double *dq = nullptr, *dout = nullptr;
  int *dst = nullptr;
  int rc = TLR_OK;
  if (up(&dq, q, (size_t)np * 50) || up<double>(&dout, nullptr, (size_t)np * 275) ||
      up<int>(&dst, nullptr, np)) {
    rc = TLR_ERR_CUDA;
  } else {
    PointParams p{np, r->reynolds, r->prandtl, r->mach, r->gamma,
                  r->sutherland_constant / r->reference_temperature};
    { k_lns_points<<<(np + 63) / 64, 64>>>(p, dq, dout, dst); count_launches(); }
    if (cudaMemcpy(blocks, dout, sizeof(double) * np * 275, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(status, dst, sizeof(int) * np, cudaMemcpyDeviceToHost))
      rc = TLR_ERR_CUDA;
  }
  cudaFree(dq); cudaFree(dout); cudaFree(dst);
  return rc;
}

extern "C" int tlr_transform_points(int np, const double *alpha, const double *phys,
                                    const double *metrics, double *fourier,
                                    double *curvilinear, int *status) {
  if (np <= 0 || !alpha || !phys || !metrics || !fourier || !curvilinear || !status)
    return TLR_ERR_ARG;
  double *da = nullptr, *dp = nullptr, *dm = nullptr, *df = nullptr, *dc = nullptr;
  int *dst = nullptr;
  int rc = TLR_OK;
  if (up(&da, alpha, (size_t)np * 2) || up(&dp, phys, (size_t)np * 275) ||
      up(&dm, metrics, (size_t)np * 10) || up<double>(&df, nullptr, (size_t)np * 350) ||
      up<double>(&dc, nullptr, (size_t)np * 350) || up<int>(&dst, nullptr, np)) {
    rc = TLR_ERR_CUDA;
  } else {
    { k_transform_points<<<(np + 63) / 64, 64>>>(np, da, dp, dm, df, dc, dst); count_launches(); }
    if (cudaMemcpy(fourier, df, sizeof(double) * np * 350, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(curvilinear, dc, sizeof(double) * np * 350, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(status, dst, sizeof(int) * np, cudaMemcpyDeviceToHost))
      rc = TLR_ERR_CUDA;
  }
  cudaFree(da); cudaFree(dp); cudaFree(dm); cudaFree(df); cudaFree(dc); cudaFree(dst);
  return rc;
}
