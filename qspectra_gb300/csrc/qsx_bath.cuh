// Debye bath one-sided correlation function on the device (FP64).
//
// Reference: DebyeBath.corr_func_complex (qspectra/bath.py:84-102)
//   C(x) = λγ [ (cot(γ/2T) − i)/(γ − i x) + 4T Σ_{k=0}^{K-1} ν_k / ((ν_k² − γ²)(ν_k − i x)) ],
//   ν_k = 2πkT, C(0) = λ(2T/γ − i),
// and Bath.corr_func_real (qspectra/bath.py:17-31) for discard_imag_corr.
//
// The truncated Matsubara sum is evaluated in closed form instead of term by
// term, which matters on GB300 where FP64 throughput is scarce.  With
// c = 2πT, a = γ/c, b = i x / c, partial fractions give
//   ν_k/((ν_k²−γ²)(ν_k−ix)) = c⁻² [ A/(k−a) + B/(k+a) + D/(k−b) ],
//   A = 1/(2(a−b)),  B = −1/(2(a+b)),  D = −b/((a−b)(a+b)),
// and Σ_{k=1}^{K−1} 1/(k−z) = ψ(K−z) − ψ(1−z).  The two real sums
// (z = ±a) depend only on (T, γ) and come in as constants fa, fb; the
// x-dependent one adds its first 7 terms directly and takes the rest from
// psi(K - iy) - psi(8 - iy), both from the Stirling-type asymptotic series
// with Bernoulli numbers B2..B14 (|z| >= 8).
#pragma once
#include "qsx_common.cuh"

namespace qsx {

struct DebyeParams {
  double T, lam, gamma;
  double cot_term;  // 1 / tan(gamma / (2T))
  double fa, fb;    // sum_{k=1}^{K-1} 1/(k - a), 1/(k + a)
  int matsubara;    // K: terms of the reference sum including k = 0
  int real_only;    // discard_imag_corr
};

__device__ __forceinline__ double2 clog_(double2 z) {
  return cmk(log(hypot(z.x, z.y)), atan2(z.y, z.x));
}

// psi(z) for |z| >= 8 from ln z - 1/(2z) - sum_{n=1..7} B_2n / (2n z^2n); the
// first omitted term is below 2e-15 relative at |z| = 8.
__device__ __forceinline__ double2 digamma_asymptotic(double2 z) {
  const double c1 = 1.0 / 12.0, c2 = -1.0 / 120.0, c3 = 1.0 / 252.0,
               c4 = -1.0 / 240.0, c5 = 1.0 / 132.0, c6 = -691.0 / 32760.0,
               c7 = 1.0 / 12.0;
  double2 zi = crecip(z);
  double2 zi2 = cmul(zi, zi);
  double2 s = cmk(c7, 0.0);
  s = cadd(cmul(s, zi2), cmk(c6, 0.0));
  s = cadd(cmul(s, zi2), cmk(c5, 0.0));
  s = cadd(cmul(s, zi2), cmk(c4, 0.0));
  s = cadd(cmul(s, zi2), cmk(c3, 0.0));
  s = cadd(cmul(s, zi2), cmk(c2, 0.0));
  s = cadd(cmul(s, zi2), cmk(c1, 0.0));
  s = cmul(s, zi2);
  return csub(csub(clog_(z), cscale(zi, 0.5)), s);
}

// sum_{k=1}^{K-1} 1/(k - i y) = sum_{k<8} (k + i y)/(k^2 + y^2)
//                              + psi(K - i y) - psi(8 - i y)   (K >= 9).
__device__ __forceinline__ double2 harmonic_shifted(int K, double y) {
  double2 head = cmk(0.0, 0.0);
  const int kmax = K < 9 ? K : 8;
  for (int k = 1; k < kmax; ++k) {
    const double inv = 1.0 / fma((double)k, (double)k, y * y);
    head.x = fma((double)k, inv, head.x);
    head.y = fma(y, inv, head.y);
  }
  if (K < 9) return head;
  return cadd(head, csub(digamma_asymptotic(cmk((double)K, -y)),
                         digamma_asymptotic(cmk(8.0, -y))));
}

// Matsubara part S(x) = sum_{k=1}^{K-1} nu_k / ((nu_k^2 - g^2)(nu_k - i x)),
// nu_k = 2 pi k T, in closed form; S(-x) = conj(S(x)).
__device__ __forceinline__ double2 debye_matsubara(const DebyeParams& p, double x) {
  const double c = 2.0 * M_PI * p.T;
  const double a = p.gamma / c;
  const double2 b = cmk(0.0, x / c);
  const double2 amb = cmk(a - b.x, -b.y);  // a - b
  const double2 apb = cmk(a + b.x, b.y);   // a + b
  const double2 A = cscale(crecip(amb), 0.5);
  const double2 B = cscale(crecip(apb), -0.5);
  const double2 D = cscale(cdiv(b, cmul(amb, apb)), -1.0);
  const double2 g = harmonic_shifted(p.matsubara, x / c);
  double2 S = cadd(cadd(cscale(A, p.fa), cscale(B, p.fb)), cmul(D, g));
  return cscale(S, 1.0 / (c * c));
}

__device__ __forceinline__ double2 debye_real(const DebyeParams& p, double x) {
  if (x == 0.0) return cmk(p.T * 2.0 * p.lam / p.gamma, 0.0);
  // J(x) = 2λγx/(γ²+x²) is odd, so J_anti(x) = J(x) for both signs.
  double J = 2.0 * p.lam * p.gamma * x / (p.gamma * p.gamma + x * x);
  return cmk((1.0 / expm1(x / p.T) + 1.0) * J, 0.0);
}

// C(x) from its Matsubara part.
__device__ __forceinline__ double2 debye_from_matsubara(const DebyeParams& p, double x,
                                                        double2 S) {
  const double2 first = cdiv(cmk(p.cot_term, -1.0), cmk(p.gamma, -x));
  return cscale(cadd(first, cscale(S, 4.0 * p.T)), p.lam * p.gamma);
}

__device__ __forceinline__ double2 debye_corr(const DebyeParams& p, double x) {
  if (p.real_only) return debye_real(p, x);
  if (x == 0.0) return cmk(p.lam * (2.0 * p.T / p.gamma), -p.lam);
  return debye_from_matsubara(p, x, debye_matsubara(p, x));
}

// C(x) and C(-x) sharing one Matsubara evaluation.
__device__ __forceinline__ void debye_corr_pair(const DebyeParams& p, double x, double2& cpos,
                                                double2& cneg) {
  if (p.real_only) {
    cpos = debye_real(p, x);
    cneg = debye_real(p, -x);
    return;
  }
  if (x == 0.0) {
    cpos = cneg = cmk(p.lam * (2.0 * p.T / p.gamma), -p.lam);
    return;
  }
  const double2 S = debye_matsubara(p, x);
  cpos = debye_from_matsubara(p, x, S);
  cneg = debye_from_matsubara(p, -x, cconj(S));
}

// Single-precision form of the same closed form, for builds whose generator
// feeds the FP32 split-word propagation: the series, logarithm and arctangent
// evaluated in FP32 (relative error a few units in 1e-7).
__device__ __forceinline__ float2 digamma_asymptotic_f(float2 z) {
  const float c1 = 1.0f / 12.0f, c2 = -1.0f / 120.0f, c3 = 1.0f / 252.0f,
              c4 = -1.0f / 240.0f, c5 = 1.0f / 132.0f, c6 = -691.0f / 32760.0f,
              c7 = 1.0f / 12.0f;
  const float2 zi = crecip(z);
  const float2 zi2 = cmul(zi, zi);
  float2 s = cmk(c7, 0.0f);
  s = cadd(cmul(s, zi2), cmk(c6, 0.0f));
  s = cadd(cmul(s, zi2), cmk(c5, 0.0f));
  s = cadd(cmul(s, zi2), cmk(c4, 0.0f));
  s = cadd(cmul(s, zi2), cmk(c3, 0.0f));
  s = cadd(cmul(s, zi2), cmk(c2, 0.0f));
  s = cadd(cmul(s, zi2), cmk(c1, 0.0f));
  s = cmul(s, zi2);
  const float2 lz = cmk(logf(hypotf(z.x, z.y)), atan2f(z.y, z.x));
  return csub(csub(lz, cscale(zi, 0.5f)), s);
}

// The FP32 forms' bath constants, each rounded once from the FP64
// parameters (on the host for kernels that take them as an argument, so the
// FP32 evaluation issues no FP64 instruction).
struct DebyeF {
  float c;          // 2 pi T
  float gamma, fa, fb, cot_term;
  float four_t;     // 4 T
  float lam_gamma;  // lam gamma
  float zero_re;    // lam 2T / gamma: Re C(0)
  float neg_lam;    // -lam: Im C(0)
  float lam, T;
  int matsubara, real_only;
};

__host__ __device__ __forceinline__ DebyeF debye_f(const DebyeParams& p) {
  DebyeF q;
  q.c = (float)(2.0 * M_PI * p.T);
  q.gamma = (float)p.gamma;
  q.fa = (float)p.fa;
  q.fb = (float)p.fb;
  q.cot_term = (float)p.cot_term;
  q.four_t = (float)(4.0 * p.T);
  q.lam_gamma = (float)(p.lam * p.gamma);
  q.zero_re = (float)(p.lam * (2.0 * p.T / p.gamma));
  q.neg_lam = (float)-p.lam;
  q.lam = (float)p.lam;
  q.T = (float)p.T;
  q.matsubara = p.matsubara;
  q.real_only = p.real_only;
  return q;
}

__device__ __forceinline__ float2 debye_matsubara_f(const DebyeF& p, float x) {
  const float c = p.c;
  const float a = p.gamma / c;
  const float y = x / c;
  const float2 amb = cmk(a, -y), apb = cmk(a, y);
  const float2 A = cscale(crecip(amb), 0.5f);
  const float2 B = cscale(crecip(apb), -0.5f);
  const float2 D = cscale(cdiv(cmk(0.0f, y), cmul(amb, apb)), -1.0f);
  float2 g = cmk(0.0f, 0.0f);
  const int K = p.matsubara;
  const int kmax = K < 9 ? K : 8;
  for (int k = 1; k < kmax; ++k) {
    const float inv = 1.0f / fmaf((float)k, (float)k, y * y);
    g.x = fmaf((float)k, inv, g.x);
    g.y = fmaf(y, inv, g.y);
  }
  if (K >= 9)
    g = cadd(g, csub(digamma_asymptotic_f(cmk((float)K, -y)), digamma_asymptotic_f(cmk(8.0f, -y))));
  const float2 S = cadd(cadd(cscale(A, p.fa), cscale(B, p.fb)), cmul(D, g));
  return cscale(S, 1.0f / (c * c));
}

__device__ __forceinline__ float2 debye_from_matsubara_f(const DebyeF& p, float x, float2 S) {
  const float2 first = cdiv(cmk(p.cot_term, -1.0f), cmk(p.gamma, -x));
  return cscale(cadd(first, cscale(S, p.four_t)), p.lam_gamma);
}

__device__ __forceinline__ float2 debye_real_f(const DebyeF& p, float x) {
  const float lam = p.lam, gam = p.gamma, T = p.T;
  if (x == 0.0f) return cmk(T * 2.0f * lam / gam, 0.0f);
  const float J = 2.0f * lam * gam * x / (gam * gam + x * x);
  return cmk((1.0f / expm1f(x / T) + 1.0f) * J, 0.0f);
}

__device__ __forceinline__ void debye_corr_pair_f(const DebyeF& p, float x, float2& cpos,
                                                  float2& cneg) {
  if (p.real_only) {
    cpos = debye_real_f(p, x);
    cneg = debye_real_f(p, -x);
    return;
  }
  if (x == 0.0f) {
    cpos = cneg = cmk(p.zero_re, p.neg_lam);
    return;
  }
  const float2 S = debye_matsubara_f(p, x);
  cpos = debye_from_matsubara_f(p, x, S);
  cneg = debye_from_matsubara_f(p, -x, cconj(S));
}

__device__ __forceinline__ void debye_corr_pair_f(const DebyeParams& p, float x, float2& cpos,
                                                  float2& cneg) {
  debye_corr_pair_f(debye_f(p), x, cpos, cneg);
}

// precision dispatch used by templated builds
__device__ __forceinline__ void debye_corr_pair_t(const DebyeParams& p, double x, double2& cp,
                                                  double2& cn) {
  debye_corr_pair(p, x, cp, cn);
}
__device__ __forceinline__ void debye_corr_pair_t(const DebyeParams& p, float x, float2& cp,
                                                  float2& cn) {
  debye_corr_pair_f(p, x, cp, cn);
}

// Host-side constants of the closed form (depend on T and gamma only).
inline DebyeParams make_debye(double T, double lam, double gamma, int K,
                              int real_only) {
  DebyeParams p;
  p.T = T;
  p.lam = lam;
  p.gamma = gamma;
  p.cot_term = 1.0 / tan(gamma / (2.0 * T));
  const double a = gamma / (2.0 * M_PI * T);
  double fa = 0.0, fb = 0.0;
  for (int k = 1; k < K; ++k) {
    fa += 1.0 / ((double)k - a);
    fb += 1.0 / ((double)k + a);
  }
  p.fa = fa;
  p.fb = fb;
  p.matsubara = K;
  p.real_only = real_only;
  return p;
}

}  // namespace qsx
