// tlr_lns.cuh -- pointwise compressible LNS blocks, streamwise Fourier
// factor and curvilinear chain rule, one 5x5 entry at a time.
//
// phys_entry<RC>() returns the entry (RC / 5, RC % 5) of the eleven
// physical blocks Gamma, A, B, C, D, Vxx, Vxy, Vxz, Vyy, Vyz, Vzz
// (LNSCoefficients.cpp:236-399).  Every nonzero entry is the reference's
// expression with the same operator order, so with --fmad=false the value is
// the reference's to the last bit.  Entries that are structurally zero in
// the reference are zero here, and the masks below let the transforms drop
// products with them: x + 0*y == x in IEEE arithmetic for finite y, so the
// dropped terms change nothing but the sign of a zero.
#pragma once

namespace tlr {

struct FlowPoint {  // BaseFlowPoint (LNSCoefficients.hpp:21-42), real
  double rho, U, V, W, T;
  double rhox, Ux, Vx, Wx, Tx;
  double rhoy, Uy, Vy, Wy, Ty;
  double rhoz, Uz, Vz, Wz, Tz;
  double Uxx, Vxx, Wxx, Txx;
  double Uyy, Vyy, Wyy, Tyy;
  double Uzz, Vzz, Wzz, Tzz;
  double Uxy, Vxy, Wxy;
  double Uxz, Vxz, Wxz;
  double Uyz, Vyz, Wyz;
};

struct Transport {  // derived scalars of LNSCoefficients::evaluate
  double Re, Pr, Pe, g2, mu, muT, muTT, mux, muy, muz;
};

__device__ __forceinline__ Transport transport(const FlowPoint &f, double Re,
                                               double Pr, double M,
                                               double gamma, double s) {
  Transport t;
  t.Re = Re;
  t.Pr = Pr;
  t.Pe = 1.0 / (gamma * M * M);
  t.g2 = 1.0 / ((gamma - 1.0) * M * M);
  const double T = f.T;
  t.mu = T * sqrt(T) * (1.0 + s) / (T + s);
  t.muT = t.mu * (1.5 / T - 1.0 / (T + s));
  t.muTT = t.muT * (1.5 / T - 1.0 / (T + s)) -
           t.mu * (1.5 / (T * T) - 1.0 / ((T + s) * (T + s)));
  t.mux = t.muT * f.Tx;
  t.muy = t.muT * f.Ty;
  t.muz = t.muT * f.Tz;
  return t;
}

// Structural masks over the 25 entries (bit r*5+c).
constexpr unsigned kDiag14 = (1u << 6) | (1u << 12) | (1u << 18) | (1u << 24);
constexpr unsigned kVyzMask = (1u << 13) | (1u << 17);
constexpr unsigned kVxyMask = (1u << 7) | (1u << 11);
constexpr unsigned kVxzMask = (1u << 8) | (1u << 16);
constexpr unsigned kViscMask = kDiag14 | kVyzMask;  // Vyy | Vzz | Vyz

struct Entry {
  double G, A, B, C, D, Vxx, Vxy, Vxz, Vyy, Vyz, Vzz;
};

template <int RC>
__device__ __forceinline__ Entry phys_entry(const FlowPoint &f,
                                            const Transport &t) {
  constexpr double t1 = 1.0 / 3.0, t2 = 2.0 / 3.0, t4 = 4.0 / 3.0;
  const double rho = f.rho, U = f.U, V = f.V, W = f.W, T = f.T;
  const double Re = t.Re, Pe = t.Pe, g2 = t.g2, mu = t.mu, muT = t.muT,
               muTT = t.muTT, mux = t.mux, muy = t.muy, muz = t.muz;
  const double Pr = t.Pr;
  Entry e{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if constexpr (RC == 0) {
    e.G = 1.0; e.A = U; e.B = V; e.C = W; e.D = f.Ux + f.Vy + f.Wz;
  } else if constexpr (RC == 1) {
    e.A = rho; e.D = f.rhox;
  } else if constexpr (RC == 2) {
    e.B = rho; e.D = f.rhoy;
  } else if constexpr (RC == 3) {
    e.C = rho; e.D = f.rhoz;
  } else if constexpr (RC == 5) {
    e.A = Pe * T;
    e.D = U * f.Ux + V * f.Uy + W * f.Uz + Pe * f.Tx;
  } else if constexpr (RC == 6) {
    e.G = rho;
    e.A = rho * U - t4 * mux / Re;
    e.B = rho * V - muy / Re;
    e.C = rho * W - muz / Re;
    e.D = rho * f.Ux;
    e.Vxx = t4 * mu / Re; e.Vyy = mu / Re; e.Vzz = mu / Re;
  } else if constexpr (RC == 7) {
    e.A = -muy / Re; e.B = t2 * mux / Re; e.D = rho * f.Uy;
    e.Vxy = t1 * mu / Re;
  } else if constexpr (RC == 8) {
    e.A = -muz / Re; e.C = t2 * mux / Re; e.D = rho * f.Uz;
    e.Vxz = t1 * mu / Re;
  } else if constexpr (RC == 9) {
    e.A = Pe * rho - muT / Re * (t4 * f.Ux - t2 * f.Vy - t2 * f.Wz);
    e.B = -muT * (f.Uy + f.Vx) / Re;
    e.C = -muT * (f.Wx + f.Uz) / Re;
    e.D = Pe * f.rhox -
          (muTT * f.Tx * t2 * (2.0 * f.Ux - f.Vy - f.Wz) +
           muTT * f.Ty * (f.Uy + f.Vx) + muTT * f.Tz * (f.Wx + f.Uz) +
           muT * (t4 * f.Uxx + f.Uyy + f.Uzz + t1 * f.Vxy + t1 * f.Wxz)) / Re;
  } else if constexpr (RC == 10) {
    e.B = Pe * T;
    e.D = U * f.Vx + V * f.Vy + W * f.Vz + Pe * f.Ty;
  } else if constexpr (RC == 11) {
    e.A = t2 * muy / Re; e.B = -mux / Re; e.D = rho * f.Vx;
    e.Vxy = t1 * mu / Re;
  } else if constexpr (RC == 12) {
    e.G = rho;
    e.A = rho * U - mux / Re;
    e.B = rho * V - t4 * muy / Re;
    e.C = rho * W - muz / Re;
    e.D = rho * f.Vy;
    e.Vxx = mu / Re; e.Vyy = t4 * mu / Re; e.Vzz = mu / Re;
  } else if constexpr (RC == 13) {
    e.B = -muz / Re; e.C = t2 * muy / Re; e.D = rho * f.Vz;
    e.Vyz = t1 * mu / Re;
  } else if constexpr (RC == 14) {
    e.A = -muT * (f.Uy + f.Vx) / Re;
    e.B = Pe * rho - muT / Re * (-t2 * f.Ux + t4 * f.Vy - t2 * f.Wz);
    e.C = -muT * (f.Vz + f.Wy) / Re;
    e.D = Pe * f.rhoy -
          (muTT * f.Tx * (f.Uy + f.Vx) +
           muTT * f.Ty * t2 * (-f.Ux + 2.0 * f.Vy - f.Wz) +
           muTT * f.Tz * (f.Vz + f.Wy) +
           muT * (f.Vxx + t4 * f.Vyy + f.Vzz + t1 * f.Uxy + t1 * f.Wyz)) / Re;
  } else if constexpr (RC == 15) {
    e.C = Pe * T;
    e.D = U * f.Wx + V * f.Wy + W * f.Wz + Pe * f.Tz;
  } else if constexpr (RC == 16) {
    e.A = t2 * muz / Re; e.C = -mux / Re; e.D = rho * f.Wx;
    e.Vxz = t1 * mu / Re;
  } else if constexpr (RC == 17) {
    e.B = t2 * muz / Re; e.C = -muy / Re; e.D = rho * f.Wy;
    e.Vyz = t1 * mu / Re;
  } else if constexpr (RC == 18) {
    e.G = rho;
    e.A = rho * U - mux / Re;
    e.B = rho * V - muy / Re;
    e.C = rho * W - t4 * muz / Re;
    e.D = rho * f.Wz;
    e.Vxx = mu / Re; e.Vyy = mu / Re; e.Vzz = t4 * mu / Re;
  } else if constexpr (RC == 19) {
    e.A = -muT * (f.Wx + f.Uz) / Re;
    e.B = -muT * (f.Vz + f.Wy) / Re;
    e.C = Pe * rho - muT / Re * (-t2 * f.Ux - t2 * f.Vy + t4 * f.Wz);
    e.D = Pe * f.rhoz -
          (muTT * f.Tx * (f.Wx + f.Uz) + muTT * f.Ty * (f.Vz + f.Wy) +
           muTT * f.Tz * t2 * (-f.Ux - f.Vy + 2.0 * f.Wz) +
           muT * (f.Wxx + f.Wyy + t4 * f.Wzz + t1 * f.Uxz + t1 * f.Vyz)) / Re;
  } else if constexpr (RC == 20) {
    e.G = -Pe * T;
    e.A = -Pe * U * T;
    e.B = -Pe * V * T;
    e.C = -Pe * W * T;
    e.D = (g2 - Pe) * (U * f.Tx + V * f.Ty + W * f.Tz);
  } else if constexpr (RC == 21) {
    e.A = -2.0 * mu * (t4 * f.Ux - t2 * f.Vy - t2 * f.Wz) / Re;
    e.B = -2.0 * mu * (f.Uy + f.Vx) / Re;
    e.C = -2.0 * mu * (f.Wx + f.Uz) / Re;
    e.D = rho * f.Tx * g2 - Pe * (rho * f.Tx + T * f.rhox);
  } else if constexpr (RC == 22) {
    e.A = -2.0 * mu * (f.Uy + f.Vx) / Re;
    e.B = -2.0 * mu * (-t2 * f.Ux + t4 * f.Vy - t2 * f.Wz) / Re;
    e.C = -2.0 * mu * (f.Vz + f.Wy) / Re;
    e.D = rho * f.Ty * g2 - Pe * (rho * f.Ty + T * f.rhoy);
  } else if constexpr (RC == 23) {
    e.A = -2.0 * mu * (f.Wx + f.Uz) / Re;
    e.B = -2.0 * mu * (f.Vz + f.Wy) / Re;
    e.C = -2.0 * mu * (-t2 * f.Ux - t2 * f.Vy + t4 * f.Wz) / Re;
    e.D = rho * f.Tz * g2 - Pe * (rho * f.Tz + T * f.rhoz);
  } else if constexpr (RC == 24) {
    e.G = rho * g2 - Pe * rho;
    e.A = rho * U * g2 - rho * U * Pe - 2.0 * f.Tx * muT * g2 / (Re * Pr);
    e.B = rho * V * g2 - rho * V * Pe - 2.0 * f.Ty * muT * g2 / (Re * Pr);
    e.C = rho * W * g2 - rho * W * Pe - 2.0 * f.Tz * muT * g2 / (Re * Pr);
    e.D = -Pe * (U * f.rhox + V * f.rhoy + W * f.rhoz) -
          (f.Txx + f.Tyy + f.Tzz) * muT * g2 / (Re * Pr) -
          (f.Tx * f.Tx + f.Ty * f.Ty + f.Tz * f.Tz) * muTT * g2 / (Re * Pr) -
          muT * (f.Uy * f.Uy + f.Vx * f.Vx + 2.0 * f.Uy * f.Vx + f.Uz * f.Uz +
                 f.Wx * f.Wx + 2.0 * f.Uz * f.Wx + f.Vz * f.Vz + f.Wy * f.Wy +
                 2.0 * f.Vz * f.Wy) / Re -
          muT * t4 * (f.Ux * f.Ux + f.Vy * f.Vy + f.Wz * f.Wz - f.Ux * f.Wz -
                      f.Ux * f.Vy - f.Vy * f.Wz) / Re;
    e.Vxx = mu * g2 / (Re * Pr); e.Vyy = mu * g2 / (Re * Pr);
    e.Vzz = mu * g2 / (Re * Pr);
  }
  return e;
}

struct Metric10 {
  double xy, xz, ey, ez, xyy, xzz, xyz, eyy, ezz, eyz;
};

struct FourierEntry {  // Gamma, K0, Ky, Kz complex; Vyy, Vyz, Vzz real
  double G, K0r, K0i, Kyr, Kyi, Kzr, Kzi, Vyy, Vyz, Vzz;
};

struct CurvEntry {  // Gamma, K0, Kxi, Keta complex; Vxixi, Vxieta, Vetaeta
  double G, K0r, K0i, Kxr, Kxi, Ker, Kei, Vxx, Vxe, Vee;
};

// StreamwiseFourier.cpp:27-37 for one entry.  ia = i*alpha, a2 = alpha^2.
template <int RC>
__device__ __forceinline__ FourierEntry fourier_entry(const Entry &p,
                                                      double ia_re,
                                                      double ia_im,
                                                      double a2_re,
                                                      double a2_im) {
  constexpr unsigned bit = 1u << RC;
  FourierEntry o;
  o.G = p.G;
  if constexpr ((kDiag14 & bit) != 0) {
    o.K0r = (p.D + ia_re * p.A) + a2_re * p.Vxx;
    o.K0i = ia_im * p.A + a2_im * p.Vxx;
  } else {
    o.K0r = p.D + ia_re * p.A;
    o.K0i = ia_im * p.A;
  }
  if constexpr ((kVxyMask & bit) != 0) {
    o.Kyr = p.B - ia_re * p.Vxy;
    o.Kyi = -(ia_im * p.Vxy);
  } else {
    o.Kyr = p.B;
    o.Kyi = 0.0;
  }
  if constexpr ((kVxzMask & bit) != 0) {
    o.Kzr = p.C - ia_re * p.Vxz;
    o.Kzi = -(ia_im * p.Vxz);
  } else {
    o.Kzr = p.C;
    o.Kzi = 0.0;
  }
  o.Vyy = p.Vyy;
  o.Vyz = p.Vyz;
  o.Vzz = p.Vzz;
  return o;
}

// CurvilinearTransform.cpp:71-94 for one entry.
template <int RC>
__device__ __forceinline__ CurvEntry curv_entry(const FourierEntry &f,
                                                const Metric10 &m) {
  constexpr unsigned bit = 1u << RC;
  CurvEntry o;
  o.G = f.G;
  o.K0r = f.K0r;
  o.K0i = f.K0i;
  o.Kxr = m.xy * f.Kyr + m.xz * f.Kzr;
  o.Ker = m.ey * f.Kyr + m.ez * f.Kzr;
  if constexpr ((kDiag14 & bit) != 0) {  // Vyy and Vzz present, Vyz zero
    o.Kxr = (o.Kxr - m.xyy * f.Vyy) - m.xzz * f.Vzz;
    o.Ker = (o.Ker - m.eyy * f.Vyy) - m.ezz * f.Vzz;
    o.Vxx = m.xy * m.xy * f.Vyy + m.xz * m.xz * f.Vzz;
    o.Vxe = 2.0 * m.xy * m.ey * f.Vyy + 2.0 * m.xz * m.ez * f.Vzz;
    o.Vee = m.ey * m.ey * f.Vyy + m.ez * m.ez * f.Vzz;
  } else if constexpr ((kVyzMask & bit) != 0) {  // only Vyz present
    o.Kxr = o.Kxr - m.xyz * f.Vyz;
    o.Ker = o.Ker - m.eyz * f.Vyz;
    o.Vxx = m.xy * m.xz * f.Vyz;
    o.Vxe = (m.xy * m.ez + m.ey * m.xz) * f.Vyz;
    o.Vee = m.ey * m.ez * f.Vyz;
  } else {
    o.Vxx = 0.0;
    o.Vxe = 0.0;
    o.Vee = 0.0;
  }
  if constexpr (((kVxyMask | kVxzMask) & bit) != 0) {
    o.Kxi = m.xy * f.Kyi + m.xz * f.Kzi;
    o.Kei = m.ey * f.Kyi + m.ez * f.Kzi;
  } else {
    o.Kxi = 0.0;
    o.Kei = 0.0;
  }
  return o;
}

// Compile-time loop over the 25 entries.
template <int RC, typename F>
__device__ __forceinline__ void for_entries(F &&fn) {
  if constexpr (RC < 25) {
    fn.template operator()<RC>();
    for_entries<RC + 1>(fn);
  }
}

}  // namespace tlr

namespace tlr {

// General (dense) forms of the two transforms for arbitrary real physical
// blocks, as exercised by the reference's transform fixtures
// (test_lns_transforms.cpp:43-65): every term of StreamwiseFourier.cpp:27-37
// and CurvilinearTransform.cpp:75-94 is kept.
__device__ __forceinline__ FourierEntry fourier_entry_full(const Entry &p,
                                                           double ia_re,
                                                           double ia_im,
                                                           double a2_re,
                                                           double a2_im) {
  FourierEntry o;
  o.G = p.G;
  o.K0r = (p.D + ia_re * p.A) + a2_re * p.Vxx;
  o.K0i = ia_im * p.A + a2_im * p.Vxx;
  o.Kyr = p.B - ia_re * p.Vxy;
  o.Kyi = -(ia_im * p.Vxy);
  o.Kzr = p.C - ia_re * p.Vxz;
  o.Kzi = -(ia_im * p.Vxz);
  o.Vyy = p.Vyy;
  o.Vyz = p.Vyz;
  o.Vzz = p.Vzz;
  return o;
}

__device__ __forceinline__ CurvEntry curv_entry_full(const FourierEntry &f,
                                                     const Metric10 &m) {
  CurvEntry o;
  o.G = f.G;
  o.K0r = f.K0r;
  o.K0i = f.K0i;
  o.Kxr = m.xy * f.Kyr + m.xz * f.Kzr - m.xyy * f.Vyy - m.xzz * f.Vzz -
          m.xyz * f.Vyz;
  o.Kxi = m.xy * f.Kyi + m.xz * f.Kzi;
  o.Ker = m.ey * f.Kyr + m.ez * f.Kzr - m.eyy * f.Vyy - m.ezz * f.Vzz -
          m.eyz * f.Vyz;
  o.Kei = m.ey * f.Kyi + m.ez * f.Kzi;
  o.Vxx = m.xy * m.xy * f.Vyy + m.xz * m.xz * f.Vzz + m.xy * m.xz * f.Vyz;
  o.Vxe = 2.0 * m.xy * m.ey * f.Vyy + 2.0 * m.xz * m.ez * f.Vzz +
          (m.xy * m.ez + m.ey * m.xz) * f.Vyz;
  o.Vee = m.ey * m.ey * f.Vyy + m.ez * m.ez * f.Vzz + m.ey * m.ez * f.Vyz;
  return o;
}

}  // namespace tlr
