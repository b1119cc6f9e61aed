// yg_valence.cu -- kernel (d): the three-layer valence chain.
//
// Forward: relative vectors with the minimum-image wrap (yaff/pes/dlist.c:
// 29-42), internal coordinates of every kind of the reference (bond, bend
// cos/angle, dihedral cos/angle and cos(n phi), Urey-Bradley, out-of-plane
// cos/angle and their means, out-of-plane distance and its square, point-line
// distance and its square; iclist.c:31-320) and the energy terms of every
// kind (vlist.c:30-155).  Back: dE/dq (vlist.c:160-265), the chain rule into
// relative-vector gradients (iclist.c:325-858) and the scatter into gpos and
// the virial (dlist.c:44-69).  One thread per row of each layer, FP64
// throughout; scatters that several rows share use FP64 atomics.
#include "yg_internal.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846;

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double *p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Gradient of a relative vector: doubles 3..5 of its 6-double row.
__device__ __forceinline__ void acc(double *row, V3 g) {
  atomicAdd(row + 3, g.x);
  atomicAdd(row + 4, g.y);
  atomicAdd(row + 5, g.z);
}

__global__ void k_dlist_fwd(const double *__restrict__ pos, const int2 *__restrict__ ij, int64_t n, CellGeom cell,
                            double *__restrict__ dl) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int i = ij[r].x, j = ij[r].y;
  double d[3] = {xsub(pos[3 * j], pos[3 * i]), xsub(pos[3 * j + 1], pos[3 * i + 1]),
                 xsub(pos[3 * j + 2], pos[3 * i + 2])};
  int m[3];
  exact_mic(d, cell, m);
  double *o = dl + 6 * r;
  o[0] = d[0]; o[1] = d[1]; o[2] = d[2];
  o[3] = 0.0; o[4] = 0.0; o[5] = 0.0;
}

// One internal-coordinate row: kind, then (delta row, sign) x 4.
struct IcRow {
  int kind;
  double *d[3];
  double s0, s1, s2;
};

__device__ __forceinline__ IcRow load_ic(const int64_t *__restrict__ row, double *dl) {
  IcRow r;
  r.kind = (int)row[0];
  for (int u = 0; u < 3; u++) r.d[u] = row[1 + 2 * u] >= 0 ? dl + 6 * row[1 + 2 * u] : dl;
  r.s0 = (double)row[2];
  r.s1 = (double)row[4];
  r.s2 = (double)row[6];
  return r;
}

__device__ __forceinline__ double bend_cos(V3 a, V3 b, double sign) {
  double da = sqrt(dot(a, a)), db = sqrt(dot(b, b));
  if (da == 0 || db == 0) return 0.0;
  return sign * dot(a, b) / da / db;
}

// cos of the dihedral: angle between the components of d0 and d2 orthogonal
// to d1 (iclist.c:57-76), times the signs of d0 and d2.
__device__ __forceinline__ double dihed_cos(V3 d0, V3 d1, V3 d2, double sign) {
  double nn = dot(d1, d1);
  V3 a = d0 - d1 * (dot(d0, d1) / nn);
  V3 b = d2 - d1 * (dot(d1, d2) / nn);
  return sign * dot(a, b) / sqrt(dot(a, a)) / sqrt(dot(b, b));
}

// sin of the dihedral, (d1 x d0).d2 |d1| / |d1 x d0| / |d2 x d1|
// (iclist.c:78-109), times the three signs.
__device__ __forceinline__ double dihed_sin(V3 d0, V3 d1, V3 d2, double sign) {
  V3 a = cross(d1, d0), b = cross(d2, d1);
  return sign * dot(a, d2) * sqrt(dot(d1, d1)) / sqrt(dot(a, a)) / sqrt(dot(b, b));
}

// Signed dihedral angle: acos where |cos| < 1/2, asin of the sine otherwise
// (iclist.c:111-141).
__device__ double dihed_angle(V3 d0, V3 d1, V3 d2, double s02, double s012) {
  double c = dihed_cos(d0, d1, d2, s02), phi;
  if (fabs(c) < 0.5) {
    phi = acos(c);
    if (dot(d0, cross(d1, d2)) * s012 > 0) phi = -phi;
  } else {
    phi = asin(dihed_sin(d0, d1, d2, s012));
    if (c < 0) {
      phi = -phi;
      phi = phi > 0 ? phi - kPi : phi + kPi;
    }
  }
  return phi;
}

// cos of the angle between u2 and the plane of u0, u1 (iclist.c:143-158).
__device__ __forceinline__ double oop_cos(V3 u0, V3 u1, V3 u2) {
  V3 n = cross(u0, u1);
  double nu = dot(n, u2);
  return sqrt(1.0 - nu * nu / dot(u2, u2) / dot(n, n));
}

__device__ __forceinline__ double oop_angle(V3 u0, V3 u1, V3 u2) {
  double c = oop_cos(u0, u1, u2);
  c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
  return acos(c);
}

__device__ double ic_value(const IcRow &r) {
  V3 d0 = ld3(r.d[0]), d1 = ld3(r.d[1]), d2 = ld3(r.d[2]);
  double c, t;
  switch (r.kind) {
    case 0: case 5: return sqrt(dot(d0, d0));
    case 1: return bend_cos(d0, d1, r.s0 * r.s1);
    case 2:
      c = bend_cos(d0, d1, r.s0 * r.s1);
      c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
      return acos(c);
    case 3: return dihed_cos(d0, d1, d2, r.s0 * r.s2);
    case 4: return dihed_angle(d0, d1, d2, r.s0 * r.s2, r.s0 * r.s1 * r.s2);
    case 6: return oop_cos(d0, d1, d2);
    case 7: return (oop_cos(d0, d1, d2) + oop_cos(d2, d0, d1) + oop_cos(d1, d2, d0)) / 3;
    case 8: return oop_angle(d0, d1, d2);
    case 9: return (oop_angle(d0, d1, d2) + oop_angle(d2, d0, d1) + oop_angle(d1, d2, d0)) / 3;
    case 10: case 11: {
      V3 n = cross(d0, d1);
      double nn = sqrt(dot(n, n));
      if (nn == 0) return 0.0;
      t = dot(n, d2) / nn;
      return r.kind == 10 ? t * r.s0 * r.s1 * r.s2 : t * t;
    }
    case 12: c = dihed_cos(d0, d1, d2, r.s0 * r.s2); return 2.0 * c * c - 1.0;
    case 13: c = dihed_cos(d0, d1, d2, r.s0 * r.s2); return c * (4.0 * c * c - 3.0);
    case 14: c = dihed_cos(d0, d1, d2, r.s0 * r.s2); c *= c; return 8.0 * c * (c - 1.0) + 1.0;
    case 15: c = dihed_cos(d0, d1, d2, r.s0 * r.s2); c *= 2.0 * c; return c * (4.0 * c * (c - 3.0) + 9.0) - 1.0;
    case 16: case 17: {
      V3 n = cross(d0, d1);
      t = dot(n, n) / dot(d2, d2);
      if (r.kind == 17) return t;
      return sqrt(t < 0 ? 0.0 : t);
    }
    default: return 0.0;
  }
}

__global__ void k_ic_fwd(const int64_t *__restrict__ ic, int64_t n, double *__restrict__ dl,
                         double *__restrict__ icv) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  IcRow row = load_ic(ic + 9 * r, dl);
  icv[2 * r] = ic_value(row);
  icv[2 * r + 1] = 0.0;
}

// Energy and dE/dq of one term (vlist.c:30-144, :160-258).  q0, q1: the
// values of the term's coordinates; g1 only for the cross term.
__device__ double term_eval(int kind, const double *__restrict__ p, double q0, double q1, double &g0, double &g1) {
  double x, x2, K, y;
  g1 = 0.0;
  switch (kind) {
    case 0:
      x = q0 - p[1];
      g0 = p[0] * x;
      return 0.5 * p[0] * x * x;
    case 1:
      g0 = p[0] + q0 * (2.0 * p[1] + q0 * (3.0 * p[2] + q0 * 4.0 * p[3]));
      return q0 * (p[0] + q0 * (p[1] + q0 * (p[2] + q0 * p[3])));
    case 2:
      x = p[1] / q0;
      g0 = p[0] * p[1] * (x * x - x * x * x);
      return 0.5 * p[0] * p[1] * p[1] * (1.0 + x * (x - 2.0));
    case 3:
      g0 = p[0] * (q1 - p[2]);
      g1 = p[0] * (q0 - p[1]);
      return p[0] * (q0 - p[1]) * (q1 - p[2]);
    case 4: {
      double s, c;
      sincos(p[0] * (q0 - p[2]), &s, &c);
      g0 = 0.5 * p[1] * p[0] * s;
      return 0.5 * p[1] * (1 - c);
    }
    case 5:
      g0 = 0.5 * p[0] * p[1];
      return 0.5 * p[0] * (1 + p[1] * q0);
    case 6:
      g0 = p[1] * 2.0 * p[0] * q0;
      return 0.5 * p[0] * (1 + p[1] * (2 * q0 * q0 - 1));
    case 7:
      g0 = p[1] * 1.5 * p[0] * (4 * q0 * q0 - 1);
      return 0.5 * p[0] * (1 + p[1] * q0 * (4 * q0 * q0 - 3));
    case 8:
      x = q0 * q0;
      g0 = p[1] * 8 * p[0] * q0 * (2 * x - 1);
      return 0.5 * p[0] * (1 + p[1] * (8 * x * x - 8 * x + 1));
    case 9:
      x = q0 * q0;
      g0 = p[1] * 6 * p[0] * q0 * (16 * x * x - 16 * x + 3);
      return 0.5 * p[0] * (1 + p[1] * (32 * x * x * x - 48 * x * x + 18 * x - 1));
    case 10:
      g0 = p[0] + q0 * (2.0 * p[1] + q0 * (3.0 * p[2] + q0 * (4.0 * p[3] + q0 * (5.0 * p[4] + q0 * 6.0 * p[5]))));
      return q0 * (p[0] + q0 * (p[1] + q0 * (p[2] + q0 * (p[3] + q0 * (p[4] + q0 * p[5])))));
    case 11:
      x = q0 - p[1];
      x2 = x * x;
      g0 = p[0] * (x - 2.024103 * x2 + 2.124366 * x2 * x);
      return 0.5 * p[0] * x2 * (1.0 - 1.349402 * x + 1.062183 * x2);
    case 12:
      x = q0 - p[1];
      x2 = x * x;
      g0 = p[0] * (x - 1.203211 * x2 + 0.367674 * x2 * x - 0.329159 * x2 * x2 + 0.711270 * x2 * x2 * x);
      return 0.5 * p[0] * x2 * (1.0 - 0.802141 * x + 0.183837 * x2 - 0.131664 * x2 * x + 0.237090 * x2 * x2);
    case 13:
      K = (p[1] - p[2]) * (p[1] - p[2]);
      K = p[0] / (K * K);
      x = q0 - p[1];
      x2 = q0 - p[2];
      y = x2 * x2;  // E = K/(2 (r1 - r2)^4) (q - r1)^2 (q - r2)^4
      g0 = K * x * y * (y + 2.0 * x * x2);
      return 0.5 * K * x * x * y * y;
    case 14: {
      double e1 = exp(-p[1] * (q0 - p[2]));
      g0 = -2.0 * p[1] * p[0] * (e1 * e1 - e1);
      return p[0] * (e1 * e1 - 2.0 * e1);
    }
    case 15:
      x = q0 - p[5];
      g0 = p[1] + x * (2.0 * p[2] + x * (3.0 * p[3] + x * 4.0 * p[4]));
      return p[0] + x * (p[1] + x * (p[2] + x * (p[3] + x * p[4])));
    default:
      g0 = 0.0;
      return 0.0;
  }
}

__global__ void k_v_fwd(const double *__restrict__ par, const int4 *__restrict__ vk, int64_t n,
                        double *__restrict__ icv, double *__restrict__ partial, int want_grad) {
  __shared__ double red[8];
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = 0.0;
  if (t < n) {
    int4 k = vk[t];  // kind, ic0, ic1
    double p[6];
#pragma unroll
    for (int u = 0; u < 6; u++) p[u] = par[6 * t + u];
    double q0 = icv[2 * k.y], q1 = k.z >= 0 ? icv[2 * k.z] : 0.0, g0, g1;
    e = term_eval(k.x, p, q0, q1, g0, g1);
    if (want_grad) {
      atomicAdd(icv + 2 * k.y + 1, g0);
      if (k.z >= 0) atomicAdd(icv + 2 * k.z + 1, g1);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    partial[blockIdx.x] = s;
  }
}

// --- back: dE/dq -> relative-vector gradients (iclist.c:325-858) ---

__device__ void back_bendcos(double *ra, double *rb, double sign, double value, double grad) {
  V3 a = ld3(ra), b = ld3(rb);
  double da = sqrt(dot(a, a)), db = sqrt(dot(b, b));
  V3 ea = a * (1.0 / da), eb = b * (1.0 / db);
  grad *= sign;
  value *= sign;
  acc(ra, (eb - ea * value) * (grad / da));
  acc(rb, (ea - eb * value) * (grad / db));
}

// d cos / d(d0, d1, d2) through the projections a = d0 - d1 (d0.d1)/|d1|^2,
// b = d2 - d1 (d1.d2)/|d1|^2 (iclist.c:366-439).  value = the signed cosine.
__device__ void back_dihed_cos(double *r0, double *r1, double *r2, double sign, double value, double grad) {
  V3 d0 = ld3(r0), d1 = ld3(r1), d2 = ld3(r2);
  double nn = dot(d1, d1);
  double p0 = dot(d0, d1), p2 = dot(d1, d2);
  V3 a = d0 - d1 * (p0 / nn), b = d2 - d1 * (p2 / nn);
  double na = sqrt(dot(a, a)), nb = sqrt(dot(b, b));
  value *= sign;
  grad *= sign;
  V3 ga = (b * (1.0 / nb) - a * (value / na)) * (1.0 / na);
  V3 gb = (a * (1.0 / na) - b * (value / nb)) * (1.0 / nb);
  double ga1 = dot(ga, d1), gb1 = dot(gb, d1);
  // a and b depend on d0 / d2 through (I - d1 d1^T / |d1|^2); on d1 through
  // -(p I + d1 d^T) / |d1|^2 + 2 p d1 d1^T / |d1|^4 (d = d0 or d2).
  acc(r0, (ga - d1 * (ga1 / nn)) * grad);
  acc(r2, (gb - d1 * (gb1 / nn)) * grad);
  V3 g1 = (ga * p0 + gb * p2 + d0 * ga1 + d2 * gb1) * (-1.0 / nn) + d1 * (2.0 * (p0 * ga1 + p2 * gb1) / (nn * nn));
  acc(r1, g1 * grad);
}

// d sin / d(d0, d1, d2) for sin = (d1 x d0).d2 |d1| / |d1 x d0| / |d2 x d1|
// (iclist.c:441-510).  value = the signed sine.
__device__ void back_dihed_sin(double *r0, double *r1, double *r2, double sign, double value, double grad) {
  V3 d0 = ld3(r0), d1 = ld3(r1), d2 = ld3(r2);
  V3 a = cross(d1, d0), b = cross(d2, d1), c = cross(d0, d2);
  double n1 = sqrt(dot(d1, d1)), ra2 = dot(a, a), rb2 = dot(b, b);
  value *= sign;
  grad *= sign;
  double ft = grad * n1 / sqrt(ra2) / sqrt(rb2);
  double f1 = grad * value / (n1 * n1), fa = grad * value / ra2, fb = grad * value / rb2;
  acc(r0, b * ft - cross(a, d1) * fa);
  acc(r1, c * ft + d1 * f1 + cross(a, d0) * fa - cross(b, d2) * fb);
  acc(r2, a * ft + cross(b, d1) * fb);
}

// d oop-cos / d(u0, u1, u2) (iclist.c:543-622); value = cos, nonzero.
__device__ void back_oop_cos(double *r0, double *r1, double *r2, double value, double grad) {
  V3 d0 = ld3(r0), d1 = ld3(r1), d2 = ld3(r2);
  V3 n = cross(d0, d1);
  double nsq = dot(n, n), usq = dot(d2, d2), nu = dot(n, d2);
  double f = -nu / usq / nsq / value * grad;
  double t1 = nu / nsq, t2 = nu / usq;
  acc(r0, (cross(d1, d2) - cross(d1, n) * t1) * f);
  acc(r1, (cross(d2, d0) - cross(n, d0) * t1) * f);
  acc(r2, (n - d2 * t2) * f);
}

__device__ void back_oop_angle(double *r0, double *r1, double *r2, double value, double grad) {
  double s, c;
  sincos(value, &s, &c);
  back_oop_cos(r0, r1, r2, c, s != 0.0 ? -grad / s : s);
}

// Signed out-of-plane distance (fac = grad sign / |n|) or its square
// (fac = 2 (n.d2) grad / |n|^2) (iclist.c:674-754).
__device__ void back_oop_dist(double *r0, double *r1, double *r2, bool squared, double sign, double grad) {
  V3 d0 = ld3(r0), d1 = ld3(r1), d2 = ld3(r2);
  V3 n = cross(d0, d1);
  double nn2 = dot(n, n), nn = sqrt(nn2), nd = dot(n, d2);
  double fac = squared ? 2 * nd * grad / nn2 : grad * sign / nn;
  double t0 = nd / nn2;
  acc(r0, (cross(d1, d2) - cross(d1, n) * t0) * fac);
  acc(r1, (cross(d2, d0) - cross(n, d0) * t0) * fac);
  acc(r2, n * fac);
}

// Squared point-line distance |d0 x d1|^2 / |d2|^2 (iclist.c:800-833).
__device__ void back_pl_sq(double *r0, double *r1, double *r2, double grad) {
  V3 d0 = ld3(r0), d1 = ld3(r1), d2 = ld3(r2);
  V3 n = cross(d0, d1);
  double usq = dot(d2, d2);
  double f = 2.0 * grad / usq;
  acc(r0, cross(d1, n) * f);
  acc(r1, cross(d0, n) * (-f));
  acc(r2, d2 * (-2.0 * grad * dot(n, n) / (usq * usq)));
}

__global__ void k_ic_back(const int64_t *__restrict__ ic, int64_t n, double *__restrict__ dl,
                          const double *__restrict__ icv) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  IcRow r = load_ic(ic + 9 * i, dl);
  double value = icv[2 * i], grad = icv[2 * i + 1];
  if (grad == 0.0) return;  // a coordinate no term depends on contributes nothing
  double *r0 = r.d[0], *r1 = r.d[1], *r2 = r.d[2];
  const double s01 = r.s0 * r.s1, s02 = r.s0 * r.s2, s012 = r.s0 * r.s1 * r.s2;
  switch (r.kind) {
    case 0: case 5:
      acc(r0, ld3(r0) * (grad / value));
      break;
    case 1: back_bendcos(r0, r1, s01, value, grad); break;
    case 2: {
      double s, c;
      sincos(value, &s, &c);
      back_bendcos(r0, r1, s01, c, -grad / s);
      break;
    }
    case 3: back_dihed_cos(r0, r1, r2, s02, value, grad); break;
    case 4: {
      V3 d0 = ld3(r0), d1 = ld3(r1), d2 = ld3(r2);
      double c = dihed_cos(d0, d1, d2, s02);
      if (fabs(c) < 0.5) {
        double t = grad / -sqrt(1 - c * c);
        if (dot(d0, cross(d1, d2)) * s012 > 0) t = -t;
        back_dihed_cos(r0, r1, r2, s02, c, t);
      } else {
        back_dihed_sin(r0, r1, r2, s012, dihed_sin(d0, d1, d2, s012), grad / c);
      }
      break;
    }
    case 6: back_oop_cos(r0, r1, r2, value, grad); break;
    case 8: back_oop_angle(r0, r1, r2, value, grad); break;
    case 7: case 9: {
      double *rot[3][3] = {{r0, r1, r2}, {r2, r0, r1}, {r1, r2, r0}};
      for (int k = 0; k < 3; k++) {
        V3 u0 = ld3(rot[k][0]), u1 = ld3(rot[k][1]), u2 = ld3(rot[k][2]);
        if (r.kind == 7)
          back_oop_cos(rot[k][0], rot[k][1], rot[k][2], oop_cos(u0, u1, u2), grad / 3.0);
        else
          back_oop_angle(rot[k][0], rot[k][1], rot[k][2], oop_angle(u0, u1, u2), grad / 3.0);
      }
      break;
    }
    case 10: back_oop_dist(r0, r1, r2, false, s012, grad); break;
    case 11: back_oop_dist(r0, r1, r2, true, 1.0, grad); break;
    case 12: case 13: case 14: case 15: {
      double c = dihed_cos(ld3(r0), ld3(r1), ld3(r2), s02), c2 = c * c, t;
      if (r.kind == 12) t = 4.0 * c;
      else if (r.kind == 13) t = 12.0 * c2 - 3.0;
      else if (r.kind == 14) t = 16.0 * c * (2.0 * c2 - 1.0);
      else t = 12.0 * c * (16.0 * c2 * (c2 - 1.0) + 3.0);
      back_dihed_cos(r0, r1, r2, s02, c, t * grad);
      break;
    }
    case 16: back_pl_sq(r0, r1, r2, value == 0.0 ? 0.0 : 0.5 * grad / value); break;
    case 17: back_pl_sq(r0, r1, r2, grad); break;
    default: break;
  }
}

__global__ void k_dlist_back(const int2 *__restrict__ ij, int64_t n, const double *__restrict__ dl,
                             double *__restrict__ gpos, double *__restrict__ partial) {
  __shared__ double red[8][9];
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (r < n) {
    const double *o = dl + 6 * r;
    int i = ij[r].x, j = ij[r].y;
    for (int k = 0; k < 3; k++) {
      atomicAdd(gpos + 3 * j + k, o[3 + k]);
      atomicAdd(gpos + 3 * i + k, -o[3 + k]);
    }
    // vtens[3*b + a] += g_a d_b (yaff/pes/dlist.c:59-67)
    for (int b = 0; b < 3; b++)
      for (int a = 0; a < 3; a++) v[3 * b + a] = o[3 + a] * o[b];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    v[q] = x;
  }
  if (lane == 0)
    for (int q = 0; q < 9; q++) red[wid][q] = v[q];
  __syncthreads();
  if (threadIdx.x < 9) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 9 + threadIdx.x] = s;
  }
}

__global__ void k_store_valence_ev(const double *__restrict__ esum, const double *__restrict__ vsum, int have_v,
                                   double *__restrict__ ev) {
  if (threadIdx.x != 0) return;
  ev[0] = esum[0];
  for (int q = 0; q < 9; q++) ev[1 + q] = have_v ? vsum[q] : 0.0;
}

}  // namespace

int yg_launch_valence(yg_ctx *ctx, int want_grad) {
  const int64_t N = ctx->natom;
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_VALENCE * N * 3;
  double *ev = ctx->d_part_ev + 10 * YG_PART_VALENCE;
  YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
  if (ctx->nterm == 0) {
    YG_CUDA(cudaMemsetAsync(ev, 0, 10 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_VALENCE] = 1;
    return YG_OK;
  }
  k_dlist_fwd<<<yg_blocks(ctx->ndelta, 256), 256, 0, ctx->stream>>>(ctx->d_pos, ctx->d_delta_ij, ctx->ndelta,
                                                                    ctx->cell, ctx->d_delta);
  YG_LAUNCH_CHECK(ctx, "k_dlist_fwd");
  k_ic_fwd<<<yg_blocks(ctx->nic, 256), 256, 0, ctx->stream>>>(ctx->d_ic, ctx->nic, ctx->d_delta, ctx->d_icval);
  YG_LAUNCH_CHECK(ctx, "k_ic_fwd");
  const int nbt = yg_blocks(ctx->nterm, 256);
  const int nbd = yg_blocks(ctx->ndelta, 256);
  int rc;
  size_t need = 64 + (size_t)nbt + 1 + (size_t)nbd * 9 + 9;
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_red, &ctx->red_cap, need * sizeof(double)))) return rc;
  double *ep = ctx->d_red + 64;
  double *esum = ep + nbt;
  double *vp = esum + 1;
  double *vsum = vp + (size_t)nbd * 9;
  k_v_fwd<<<nbt, 256, 0, ctx->stream>>>(ctx->d_vpar, ctx->d_vkind, ctx->nterm, ctx->d_icval, ep, want_grad);
  YG_LAUNCH_CHECK(ctx, "k_v_fwd");
  if ((rc = yg_launch_reduce_ev(ctx, ep, nbt, 1, esum))) return rc;
  if (want_grad) {
    k_ic_back<<<yg_blocks(ctx->nic, 256), 256, 0, ctx->stream>>>(ctx->d_ic, ctx->nic, ctx->d_delta, ctx->d_icval);
    YG_LAUNCH_CHECK(ctx, "k_ic_back");
    k_dlist_back<<<nbd, 256, 0, ctx->stream>>>(ctx->d_delta_ij, ctx->ndelta, ctx->d_delta, gpos, vp);
    YG_LAUNCH_CHECK(ctx, "k_dlist_back");
    if ((rc = yg_launch_reduce_ev(ctx, vp, nbd, 9, vsum))) return rc;
  }
  k_store_valence_ev<<<1, 32, 0, ctx->stream>>>(esum, vsum, want_grad, ev);
  YG_LAUNCH_CHECK(ctx, "k_store_valence_ev");
  ctx->part_valid[YG_PART_VALENCE] = 1;
  return YG_OK;
}
