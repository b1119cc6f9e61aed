// yg_pairterm.cuh -- one pair of one real-space potential (device code
// shared by the list-driven pair kernel and the MC trial kernel).
#pragma once

#include "yg_internal.cuh"

template <typename T> struct Num;
template <> struct Num<double> {
  static __device__ __forceinline__ double exp_(double x) { return exp(x); }
  static __device__ __forceinline__ double erfc_(double x) { return erfc(x); }
  static __device__ __forceinline__ double erf_(double x) { return erf(x); }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
};
template <> struct Num<float> {
  static __device__ __forceinline__ float exp_(float x) { return expf(x); }
  static __device__ __forceinline__ float erfc_(float x) { return erfcf(x); }
  static __device__ __forceinline__ float erf_(float x) { return erff(x); }
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
};

// Entry (a, b, c, d) of a type-pair table in the precision of the caller.
template <typename T> struct TabEntry;
template <> struct TabEntry<double> {
  static __device__ __forceinline__ double4_32a get(const PairPotDev &P, int k) { return P.tab64[k]; }
};
template <> struct TabEntry<float> {
  static __device__ __forceinline__ float4 get(const PairPotDev &P, int k) { return P.tab32[k]; }
};

// Kinds beyond LJ / MM3 / EI: MM3CAP and Grimme (per-atom parameters), and
// the type-pair table kinds.  Formulas of yaff/pes/pair_pot.c:373-419
// (MM3CAP, including its force below the cap, which the reference takes from
// the unmodified MM3 expression at the cap's x), :434-455 (Grimme), :473-489
// (ExpRep), :506-522 (QMDFFRep), :540-557 (LJCross), :576-629 (DampDisp with
// the Tang-Toennies damping) and :651-677 (Disp68BJDamp).
template <typename T>
__device__ __noinline__ void pair_term_more(const PairPotDev &P, T d, T d2, T pi0, T pi1, T pi3, T pj0, T pj1,
                                            T pj3, T &v, T &g) {
  typedef Num<T> M;
  if (P.kind == YG_POT_MM3CAP) {
    const T sig = pi0 + pj0, eps = pi1 * pj1;
    T x = d / sig;
    if (pi3 + pj3 == (T)0) {
      const T xmax = (T)0.355114;
      const T xc = x > xmax ? x : xmax;
      const T ex = (T)1.84e5 * M::exp_((T)-12.0 * xc);
      T x6 = xc * xc;
      x6 = x6 * x6 * x6 / (T)2.25;
      g = eps / d * ((T)-12.0 / sig * ex + (T)6.0 / d / x6);
      v = x > xmax ? eps * (ex - (T)1 / x6) : eps * ((T)5799.303156 - (T)12182.86986 * x);
    } else {
      const T ex = (T)1.84e5 * M::exp_((T)-12.0 * x);
      g = eps / d * ((T)-12.0 / sig * ex);
      v = eps * ex;
    }
    return;
  }
  if (P.kind == YG_POT_GRIMME) {
    const T r0 = pi0 + pj0, c6 = pi1 * pj1;
    const T ex = M::exp_((T)-20.0 * (d / r0 - (T)1.0));
    const T f = (T)1.0 / ((T)1.0 + ex);
    const T d6 = d2 * d2 * d2;
    const T e = (T)1.1 * f * c6 / d6;
    g = e / d * ((T)6.0 / d - (T)20.0 / r0 * f * ex);
    v = -e;
    return;
  }
  const auto t = TabEntry<T>::get(P, (int)pi0 * P.ntype + (int)pj0);
  v = (T)0;
  g = (T)0;
  switch (P.kind) {
    case YG_POT_EXPREP:
      if (t.x != (T)0 && t.y != (T)0) {
        v = t.x * M::exp_(-t.y * d);
        g = -v * t.y / d;
      }
      break;
    case YG_POT_QMDFFREP:
      if (t.x != (T)0 && t.y != (T)0) {
        v = t.x / d * M::exp_(-t.y * d);
        g = -(t.y + (T)1 / d) * v / d;
      }
      break;
    case YG_POT_LJCROSS: {
      T x = t.y / d;
      x *= x;
      x *= x * x;
      g = (T)24.0 * t.x / d2 * x * ((T)1.0 - (T)2.0 * x);
      v = (T)4.0 * t.x * (x * (x - (T)1.0));
      break;
    }
    case YG_POT_DAMPDISP: {
      if (t.x == (T)0) break;
      T dn = (T)1;
      for (int j = 0; j < P.power; j++) dn *= d;
      const T disp = -t.x / dn;
      if (t.y == (T)0) {
        v = disp;
        g = -(T)P.power * disp / d2;
      } else {
        // 1 - exp(-x) sum_{k<=n} x^k / k!, x = b d, and its x-derivative
        const T x = t.y * d;
        T term = (T)1, poly = (T)1;
        for (int k = 1; k <= P.power; k++) {
          term = term * x / (T)k;
          poly += term;
        }
        const T e = M::exp_(-x);
        const T damp = (T)1 - poly * e;
        g = (e * term * t.y - (T)P.power / d * damp) * disp / d;
        v = damp * disp;
      }
      break;
    }
    default: {  // YG_POT_DISP68BJ: (s6 c6, s8 c8, R^6, R^8)
      const T d4 = d2 * d2, d6 = d4 * d2, d8 = d4 * d4;
      const T u6 = (T)1 / (d6 + t.z), u8 = (T)1 / (d8 + t.w);
      v = -t.x * u6 - t.y * u8;
      g = (T)6.0 * t.x * u6 * u6 * d4 + (T)8.0 * t.y * u8 * u8 * d6;
      break;
    }
  }
}

// Energy v and g = (dv/dd)/d of one pair for one potential, truncation
// included.  Formulas of yaff/pes/pair_pot.c:277-301 (LJ), :321-352 (MM3),
// :711-751 (EI) and truncation.c:30-76; the other kinds in pair_term_more.
template <typename T>
__device__ __forceinline__ void pair_term(const PairPotDev &P, T rcT, T parT, T alphaT, T invdT, T d, T d2, T pi0,
                                          T pi1, T pi2, T pi3, T pj0, T pj1, T pj2, T pj3, T qi, T qj, T &v, T &g) {
  typedef Num<T> M;
  const T two_div_sqrt_pi = (T)1.1283791670955125739;
  if (P.kind > YG_POT_EI) {
    pair_term_more<T>(P, d, d2, pi0, pi1, pi3, pj0, pj1, pj3, v, g);
  } else if (P.kind == YG_POT_LJ) {
    T sig = (T)0.5 * (pi0 + pj0);
    T eps = pi1 * pj1;
    T x = sig / d;
    x *= x;
    x *= x * x;
    g = (T)24.0 * eps / d2 * x * ((T)1.0 - (T)2.0 * x);
    v = (T)4.0 * eps * (x * (x - (T)1.0));
  } else if (P.kind == YG_POT_MM3) {
    T sig = pi0 + pj0;
    T eps = pi1 * pj1;
    T x = sig / d;
    T ex = (T)1.84e5 * M::exp_((T)-12.0 / x);
    if (pi3 + pj3 == (T)0) {
      x *= x;
      x *= (T)2.25 * x * x;
      g = eps / d * ((T)-12.0 / sig * ex + (T)6.0 / d * x);
      v = eps * (ex - x);
    } else {
      g = eps / d * ((T)-12.0 / sig * ex);
      v = eps * ex;
    }
  } else {
    T qq = qi * qj * invdT;
    T alpha = alphaT;
    T rab2 = pi2 + pj2;
    if (alpha > (T)0) {
      T x = alpha * d;
      if (rab2 > (T)0) {
        T rab = M::sqrt_(rab2);
        T y = d / rab;
        v = qq / d * (M::erfc_(x) - M::erfc_(y));
        g = (two_div_sqrt_pi * (M::exp_(-y * y) / rab - M::exp_(-x * x) * alpha) * qq - v) / d2;
      } else {
        v = qq * M::erfc_(x) / d;
        g = (-two_div_sqrt_pi * alpha * M::exp_(-x * x) * qq - v) / d2;
      }
    } else {
      if (rab2 > (T)0) {
        T rab = M::sqrt_(rab2);
        T y = d / rab;
        v = qq / d * M::erf_(y);
        g = (two_div_sqrt_pi / rab * M::exp_(-y * y) * qq - v) / d2;
      } else {
        v = qq / d;
        g = -v / d2;
      }
    }
  }
  if (P.tr_kind != YG_TR_NONE && (v != (T)0 || g != (T)0)) {
    T rc = rcT, par = parT, h, hg;
    if (P.tr_kind == YG_TR_HAMMER) {
      T x = d - rc;
      h = M::exp_(par / x);
      hg = -h * par / x / x;
    } else {
      T x = rc - d;
      if (x > par) {
        h = (T)1;
        hg = (T)0;
      } else {
        x /= par;
        h = ((T)3 - (T)2 * x) * x * x;
        hg = (T)-6 * x * ((T)1 - x) / par;
      }
    }
    g = g * h + v * hg / d;
    v *= h;
  }
}

// erfc(x) for x >= 0 in FP32 from the Chebyshev-fitted form of Numerical
// Recipes (erfcc: t exp(-x^2 + P(t)), t = 1/(1 + x/2), fractional error below
// 1.2e-7 everywhere), which keeps the relative accuracy of the tail where the
// real-space Ewald term is evaluated.
static __device__ __forceinline__ float erfc_cheb(float x) {
  const float t = __frcp_rn(1.0f + 0.5f * x);  // = 1.0f / (1 + x / 2) (both correctly rounded)
  float p = 0.17087277f;
  p = fmaf(p, t, -0.82215223f);
  p = fmaf(p, t, 1.48851587f);
  p = fmaf(p, t, -1.13520398f);
  p = fmaf(p, t, 0.27886807f);
  p = fmaf(p, t, -0.18628806f);
  p = fmaf(p, t, 0.09678418f);
  p = fmaf(p, t, 0.37409196f);
  p = fmaf(p, t, 1.00002368f);
  p = fmaf(p, t, -1.26551223f);
  return t * expf(fmaf(-x, x, p));
}

// FP32 evaluation of one pair (mixed modes): one reciprocal square root per
// pair instead of divisions.  Same formulas as pair_term; Gaussian charges,
// bare Coulomb and truncation fall back to pair_term.
static __device__ __forceinline__ void pair_term_f32(const PairPotDev &P, float rcT, float parT, float alphaT, float invdT,
                                              float d, float d2, float inv_d, float pi0, float pi1, float pi2,
                                              float pi3, float pj0, float pj1, float pj2, float pj3, float qi,
                                              float qj, float &v, float &g) {
  const float inv_d2 = inv_d * inv_d;
  if (P.tr_kind == YG_TR_NONE) {
    if (P.kind == YG_POT_LJ) {
      const float sig = 0.5f * (pi0 + pj0);
      const float eps = pi1 * pj1;
      const float s2 = sig * sig * inv_d2;
      const float x = s2 * s2 * s2;
      g = 24.0f * eps * inv_d2 * x * (1.0f - 2.0f * x);
      v = 4.0f * eps * (x * (x - 1.0f));
      return;
    }
    if (P.kind == YG_POT_MM3) {
      const float sig = pi0 + pj0;
      const float eps = pi1 * pj1;
      const float inv_sig = __frcp_rn(sig);  // = 1.0f / sig (both correctly rounded)
      const float ex = 1.84e5f * expf(-12.0f * d * inv_sig);
      if (pi3 + pj3 == 0.0f) {
        const float s2 = sig * sig * inv_d2;
        const float x = 2.25f * s2 * s2 * s2;
        g = eps * inv_d * (-12.0f * inv_sig * ex + 6.0f * inv_d * x);
        v = eps * (ex - x);
      } else {
        g = eps * inv_d * (-12.0f * inv_sig * ex);
        v = eps * ex;
      }
      return;
    }
    if (P.kind == YG_POT_EI && alphaT > 0.0f && pi2 + pj2 == 0.0f) {
      const float qq = qi * qj * invdT;
      const float x = alphaT * d;
      const float e = expf(-x * x);
      v = qq * erfc_cheb(x) * inv_d;
      g = (-1.1283791670955126f * alphaT * e * qq - v) * inv_d2;
      return;
    }
  }
  pair_term<float>(P, rcT, parT, alphaT, invdT, d, d2, pi0, pi1, pi2, pi3, pj0, pj1, pj2, pj3, qi, qj, v, g);
}

