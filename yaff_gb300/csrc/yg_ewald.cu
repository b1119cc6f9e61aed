// yg_ewald.cu -- kernel (c): Ewald reciprocal-space sum and its corrections.
//
// Same half-sphere direct sum as yaff/pes/ewald.c:32-150, restructured for
// the GPU.  Write the phase of atom a at k = 2 pi (g0 b0 + g1 b1 + m b2) as
// E0[a][g0] E1[a][g1] E2[a][m] with Ei[a][g] = exp(2 pi i g s_ai) (s = the
// fractional coordinates; negative g by conjugation).  Then
//
//   S[c][m] = sum_a X[a][c] Y[a][m],  X = E0 E1 (column c = (g0, g1)),
//                                     Y = q E2
//
// is a complex matrix product over the atoms, and the gradient
//
//   dE/dr_a = -2 pi (b0 sum_c g0 Im(P_ac Z_ac) + b1 sum_c g1 Im(P_ac Z_ac)
//                     + b2 sum_c Im(P_ac Z2_ac)),
//   Z_ac = sum_m Y[a][m] conj(W[c][m]),  Z2_ac = sum_m m Y[a][m] conj(W[c][m]),
//   P_ac = X[a][c],  W = 2 A(k) S_eff(k)
//
// is a second product over m.  Both run as shared-memory tiled kernels over
// 8x8 blocks of (g0, g1) columns; blocks wholly outside the k-sphere are
// skipped.  The phases are built per atom from FP64 fractional coordinates
// (reduced to [0,1) before the sine/cosine), so FP32 tables keep ~1e-7
// absolute phase accuracy even where |k.r| reaches hundreds of radians.
// Partial structure factors of atom chunks are summed in FP64 in a fixed
// order; the energy, the virial and the prefactors are FP64.
#include <cmath>
#include <type_traits>
#include <vector>

#include "yg_internal.cuh"

namespace {

#define EW_TC 64     // columns per tile (8 x 8 in g0, g1)
#define EW_MT 32     // m values per S-pass tile
#define EW_KA 32     // atoms staged per step in the S pass
#define EW_ATB 512   // atoms per S-pass block
#define EW_MAXM 64   // largest supported G2 + 1

template <typename T> struct C2;
template <> struct C2<float> { typedef float2 t; };
template <> struct C2<double> { typedef double2 t; };

template <typename T> __device__ __forceinline__ typename C2<T>::t cmk(T a, T b) {
  typename C2<T>::t r;
  r.x = a;
  r.y = b;
  return r;
}

// Per-atom phase tables: for every atom L = (G0+1)+(G1+1)+(G2+1) complex
// values, E0[0..G0], E1[0..G1], q*E2[0..G2].
template <typename T>
__global__ void k_tables(const double *__restrict__ pos, const double *__restrict__ charge, int64_t natom,
                         CellGeom cell, int G0, int G1, int G2, typename C2<T>::t *__restrict__ tab) {
  const int L = G0 + G1 + G2 + 3;
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= natom * L) return;
  int64_t a = idx / L;
  int e = (int)(idx - a * L);
  int axis, g;
  if (e <= G0) { axis = 0; g = e; }
  else if (e <= G0 + 1 + G1) { axis = 1; g = e - G0 - 1; }
  else { axis = 2; g = e - G0 - G1 - 2; }
  const double *gv = cell.gv + 3 * axis;
  double s = gv[0] * pos[3 * a] + gv[1] * pos[3 * a + 1] + gv[2] * pos[3 * a + 2];
  s -= floor(s);
  double x = (double)g * s;
  x -= rint(x);            // x in [-0.5, 0.5]
  T sn, cs;
  if (sizeof(T) == 8) {
    double dsn, dcs;
    sincospi(2.0 * x, &dsn, &dcs);
    sn = (T)dsn;
    cs = (T)dcs;
  } else {
    float fsn, fcs;
    sincospif(2.0f * (float)x, &fsn, &fcs);
    sn = (T)fsn;
    cs = (T)fcs;
  }
  if (axis == 2) {
    T q = (T)charge[a];
    cs *= q;
    sn *= q;
  }
  tab[idx] = cmk<T>(cs, sn);
}

template <typename T>
__device__ __forceinline__ typename C2<T>::t tab_get(const typename C2<T>::t *__restrict__ row, int base, int g) {
  typename C2<T>::t v = row[base + (g < 0 ? -g : g)];
  if (g < 0) v.y = -v.y;
  return v;
}

struct Tile {
  int gb0, gb1, mhi;
};

// S pass.  grid = (tiles, atom chunks, m tiles); 128 threads, each owning
// 4 columns x 4 m values of the 64 x 32 output tile.
template <typename T, typename TA>
__global__ void __launch_bounds__(128) k_sfac(const typename C2<T>::t *__restrict__ tab, int a0, int a1, int G0,
                                              int G1, int G2, const int4 *__restrict__ tiles,
                                              typename C2<TA>::t *__restrict__ Spart, int ntile) {
  typedef typename C2<T>::t CT;
  __shared__ CT sX[EW_KA][EW_TC];
  __shared__ CT sY[EW_KA][EW_MT];
  const int L = G0 + G1 + G2 + 3;
  const int4 tl = tiles[blockIdx.x];
  const int mb = blockIdx.z * EW_MT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int abeg = a0 + blockIdx.y * EW_ATB;
  const int aend = min(a1, abeg + EW_ATB);
  T acc_re[4][4], acc_im[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      acc_re[i][j] = (T)0;
      acc_im[i][j] = (T)0;
    }
  if (mb <= tl.z) {
    for (int ab = abeg; ab < aend; ab += EW_KA) {
      // stage X (E0 E1) and Y (q E2) for EW_KA atoms
      for (int v = threadIdx.x; v < EW_KA * EW_TC; v += blockDim.x) {
        int la = v / EW_TC, c = v % EW_TC;
        int a = ab + la;
        CT x = cmk<T>((T)0, (T)0);
        int g0 = tl.x + (c >> 3), g1 = tl.y + (c & 7);
        if (a < aend && g0 <= G0 && g1 <= G1) {
          const CT *row = tab + (int64_t)a * L;
          CT e0 = tab_get<T>(row, 0, g0);
          CT e1 = tab_get<T>(row, G0 + 1, g1);
          x = cmk<T>(e0.x * e1.x - e0.y * e1.y, e0.x * e1.y + e0.y * e1.x);
        }
        sX[la][c] = x;
      }
      for (int v = threadIdx.x; v < EW_KA * EW_MT; v += blockDim.x) {
        int la = v / EW_MT, m = v % EW_MT;
        int a = ab + la;
        CT y = cmk<T>((T)0, (T)0);
        if (a < aend && mb + m <= G2) y = tab[(int64_t)a * L + G0 + G1 + 2 + mb + m];
        sY[la][m] = y;
      }
      __syncthreads();
#pragma unroll 4
      for (int la = 0; la < EW_KA; la++) {
        CT x[4], y[4];
#pragma unroll
        for (int i = 0; i < 4; i++) x[i] = sX[la][tx * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; j++) y[j] = sY[la][ty * 4 + j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            acc_re[i][j] += x[i].x * y[j].x - x[i].y * y[j].y;
            acc_im[i][j] += x[i].x * y[j].y + x[i].y * y[j].x;
          }
      }
      __syncthreads();
    }
  }
  // partial layout: [chunk][tile][mtile][c][m]
  typedef typename C2<TA>::t CA;
  int64_t base = (((int64_t)blockIdx.y * ntile + blockIdx.x) * gridDim.z + blockIdx.z) * (EW_TC * EW_MT);
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      CA v;
      v.x = (TA)acc_re[i][j];
      v.y = (TA)acc_im[i][j];
      Spart[base + (tx * 4 + i) * EW_MT + ty * 4 + j] = v;
    }
}

// Sums the chunk partials in FP64 into the dense S[c][m] grid (re, im).
template <typename TA>
__global__ void k_sfac_reduce(const typename C2<TA>::t *__restrict__ Spart, int nchunk, int ntile, int nmt,
                              const int4 *__restrict__ tiles, int G0, int G1, int nm,
                              double *__restrict__ S) {
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t per = (int64_t)ntile * nmt * EW_TC * EW_MT;
  if (idx >= per) return;
  int m = (int)(idx % EW_MT);
  int c = (int)((idx / EW_MT) % EW_TC);
  int mt = (int)((idx / (EW_MT * EW_TC)) % nmt);
  int t = (int)(idx / ((int64_t)EW_MT * EW_TC * nmt));
  int4 tl = tiles[t];
  int g0 = tl.x + (c >> 3), g1 = tl.y + (c & 7), mm = mt * EW_MT + m;
  if (g0 > G0 || g1 > G1 || mm >= nm) return;
  double re = 0.0, im = 0.0;
  for (int ch = 0; ch < nchunk; ch++) {
    typename C2<TA>::t v = Spart[(int64_t)ch * per + idx];
    re += (double)v.x;
    im += (double)v.y;
  }
  int64_t col = (int64_t)(g0 + G0) * (2 * G1 + 1) + (g1 + G1);
  S[2 * (col * nm + mm)] = re;
  S[2 * (col * nm + mm) + 1] = im;
}

// Energy and virial per k (FP64), plus the force-pass weights
// conj(W_g) = conj(2 A S_eff,g) for the atom groups in use.
template <typename T>
__global__ void k_ewald_energy(const double *__restrict__ S, int nS, int64_t nk_dense, const double *__restrict__ pref,
                               int G0, int G1, int nm, CellGeom cell, double fac2, int ngroup,
                               typename C2<T>::t *__restrict__ W, double *__restrict__ partial) {
  __shared__ double red[256 / 32][7];
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = 0.0, v[6] = {0, 0, 0, 0, 0, 0};
  if (idx < nk_dense) {
    double A = pref[idx];
    const double *S0 = S + 2 * idx;
    double c0 = S0[0], s0 = S0[1], c1 = 0, s1 = 0, c2 = 0, s2 = 0;
    if (nS == 3) {
      c1 = S[2 * (nk_dense + idx)];
      s1 = S[2 * (nk_dense + idx) + 1];
      c2 = S[2 * (2 * nk_dense + idx)];
      s2 = S[2 * (2 * nk_dense + idx) + 1];
    }
    if (A != 0.0) {
      double s = c0 * (c0 + 2.0 * (c1 + c2)) + s0 * (s0 + 2.0 * (s1 + s2));
      s += 2.0 * (c1 * c2 + s1 * s2);
      e = A * s;
      int64_t col = idx / nm;
      int m = (int)(idx - col * nm);
      int g0 = (int)(col / (2 * G1 + 1)) - G0;
      int g1 = (int)(col % (2 * G1 + 1)) - G1;
      double k[3];
      const double tp = 6.2831853071795864769;
      for (int x = 0; x < 3; x++)
        k[x] = tp * (g0 * cell.gv[x] + g1 * cell.gv[3 + x] + m * cell.gv[6 + x]);
      double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      double cc = A * 2.0 * (1.0 / ksq + fac2) * s;
      v[0] = cc * k[0] * k[0];
      v[1] = cc * k[1] * k[1];
      v[2] = cc * k[2] * k[2];
      v[3] = cc * k[0] * k[1];
      v[4] = cc * k[0] * k[2];
      v[5] = cc * k[1] * k[2];
    }
    // weights: group 0 = mid atoms (S0+S1+S2), 1 = low atoms (S0+S2),
    // 2 = high atoms (S0+S1); conj stored.
    for (int g = 0; g < ngroup; g++) {
      double wr = c0, wi = s0;
      if (g == 0) { wr += c1 + c2; wi += s1 + s2; }
      else if (g == 1) { wr += c2; wi += s2; }
      else { wr += c1; wi += s1; }
      W[(int64_t)g * nk_dense + idx] = cmk<T>((T)(2.0 * A * wr), (T)(-2.0 * A * wi));
    }
  }
  // block reduction (fixed order)
  double vals[7] = {e, v[0], v[1], v[2], v[3], v[4], v[5]};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 7; q++) {
    double x = vals[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    vals[q] = x;
  }
  if (lane == 0)
    for (int q = 0; q < 7; q++) red[wid][q] = vals[q];
  __syncthreads();
  if (threadIdx.x < 7) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 7 + threadIdx.x] = s;
  }
}

template <typename T> struct CompAcc {
  T s;
  __device__ __forceinline__ void init() { s = (T)0; }
  __device__ __forceinline__ void add(T x) { s += x; }
  __device__ __forceinline__ double value() const { return (double)s; }
};
template <> struct CompAcc<float> {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Force pass.  grid = atom tiles (16*RA atoms) of one group; 256 threads:
// ta = tid % 16 owns RA atoms, tc = tid / 16 owns 4 consecutive columns.
template <typename T, int RA>
__global__ void __launch_bounds__(256) k_ewald_force(const typename C2<T>::t *__restrict__ tab, int a0, int a1,
                                                     int G0, int G1, int G2, const int4 *__restrict__ tiles,
                                                     int ntile, const typename C2<T>::t *__restrict__ W,
                                                     double *__restrict__ gfrac) {
  typedef typename C2<T>::t CT;
  extern __shared__ unsigned char smem_raw[];
  const int NA = 16 * RA;
  const int nm = G2 + 1;
  CT *sY = reinterpret_cast<CT *>(smem_raw);          // [nm][NA]
  CT *sW = sY + (size_t)nm * NA;                       // [nm][EW_TC]
  const int L = G0 + G1 + G2 + 3;
  const int ta = threadIdx.x & 15, tc = threadIdx.x >> 4;
  const int abase = a0 + blockIdx.x * NA;
  // stage Y = q E2 for the block's atoms
  for (int v = threadIdx.x; v < nm * NA; v += blockDim.x) {
    int m = v / NA, la = v % NA;
    int a = abase + la;
    sY[v] = (a < a1) ? tab[(int64_t)a * L + G0 + G1 + 2 + m] : cmk<T>((T)0, (T)0);
  }
  CompAcc<T> acc[RA][3];
#pragma unroll
  for (int r = 0; r < RA; r++)
#pragma unroll
    for (int q = 0; q < 3; q++) acc[r][q].init();
  const int ncolrow = 2 * G1 + 1;
  for (int t = 0; t < ntile; t++) {
    const int4 tl = tiles[t];
    const int mhi = tl.z;
    __syncthreads();
    for (int v = threadIdx.x; v < (mhi + 1) * EW_TC; v += blockDim.x) {
      int m = v / EW_TC, c = v % EW_TC;
      int g0 = tl.x + (c >> 3), g1 = tl.y + (c & 7);
      CT w = cmk<T>((T)0, (T)0);
      if (g0 <= G0 && g1 <= G1) {
        int64_t col = (int64_t)(g0 + G0) * ncolrow + (g1 + G1);
        w = W[col * nm + m];
      }
      sW[m * EW_TC + c] = w;
    }
    __syncthreads();
    T zr[RA][4], zi[RA][4], z2r[RA][4], z2i[RA][4];
#pragma unroll
    for (int r = 0; r < RA; r++)
#pragma unroll
      for (int i = 0; i < 4; i++) {
        zr[r][i] = (T)0; zi[r][i] = (T)0; z2r[r][i] = (T)0; z2i[r][i] = (T)0;
      }
    for (int m = 0; m <= mhi; m++) {
      CT y[RA], w[4];
#pragma unroll
      for (int r = 0; r < RA; r++) y[r] = sY[m * NA + ta * RA + r];
#pragma unroll
      for (int i = 0; i < 4; i++) w[i] = sW[m * EW_TC + tc * 4 + i];
      const T fm = (T)m;
#pragma unroll
      for (int r = 0; r < RA; r++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          T pr = y[r].x * w[i].x - y[r].y * w[i].y;
          T pi = y[r].x * w[i].y + y[r].y * w[i].x;
          zr[r][i] += pr;
          zi[r][i] += pi;
          z2r[r][i] += fm * pr;
          z2i[r][i] += fm * pi;
        }
    }
    // epilogue: P = E0 E1 of each (atom, column)
    const int c0 = tc * 4;
    const int g0 = tl.x + (c0 >> 3);
#pragma unroll
    for (int r = 0; r < RA; r++) {
      int a = abase + ta * RA + r;
      if (a >= a1) continue;
      const CT *row = tab + (int64_t)a * L;
      if (g0 > G0) continue;
      CT e0 = tab_get<T>(row, 0, g0);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        int g1 = tl.y + ((c0 + i) & 7);
        if (g1 > G1) continue;
        CT e1 = tab_get<T>(row, G0 + 1, g1);
        T pr = e0.x * e1.x - e0.y * e1.y;
        T pi = e0.x * e1.y + e0.y * e1.x;
        T im1 = pr * zi[r][i] + pi * zr[r][i];
        T im2 = pr * z2i[r][i] + pi * z2r[r][i];
        acc[r][0].add((T)g0 * im1);
        acc[r][1].add((T)g1 * im1);
        acc[r][2].add(im2);
      }
    }
  }
  // reduce the 16 column groups of every atom in a fixed order
  __syncthreads();
  double *red = reinterpret_cast<double *>(smem_raw);  // [16][NA][3]
#pragma unroll
  for (int r = 0; r < RA; r++)
#pragma unroll
    for (int q = 0; q < 3; q++) red[((size_t)tc * NA + ta * RA + r) * 3 + q] = acc[r][q].value();
  __syncthreads();
  for (int v = threadIdx.x; v < NA * 3; v += blockDim.x) {
    int la = v / 3, q = v % 3;
    int a = abase + la;
    if (a >= a1) continue;
    double s = 0.0;
    for (int g = 0; g < 16; g++) s += red[((size_t)g * NA + la) * 3 + q];
    gfrac[(int64_t)a * 3 + q] = s;
  }
}

// gpos = -2 pi (b0 f0 + b1 f1 + b2 f2) / dielectric (orig order).
__global__ void k_ewald_gpos(const double *__restrict__ gfrac, int64_t natom, CellGeom cell, double scale,
                             double *__restrict__ gpos) {
  int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= natom) return;
  double f0 = gfrac[3 * a], f1 = gfrac[3 * a + 1], f2 = gfrac[3 * a + 2];
  for (int x = 0; x < 3; x++)
    gpos[3 * a + x] = scale * (f0 * cell.gv[x] + f1 * cell.gv[3 + x] + f2 * cell.gv[6 + x]);
}

__global__ void k_store_ewald_ev(const double *__restrict__ sums, double scale, double *__restrict__ ev) {
  if (threadIdx.x != 0) return;
  double e = sums[0];
  // vtens -= E on the diagonal, then the dielectric factor
  double v[9] = {sums[1] - e, sums[4], sums[5], sums[4], sums[2] - e, sums[6], sums[5], sums[6], sums[3] - e};
  ev[0] = e * scale;
  for (int q = 0; q < 9; q++) ev[1 + q] = v[q] * scale;
}

// Excluded-pair part of the Ewald correction (yaff/pes/ewald.c:290-335):
// one thread per scaling row, FP64, minimum image as in the reference.
__global__ void k_ewald_corr(const double *__restrict__ pos, const double *__restrict__ q, const int2 *__restrict__ ab,
                             const double *__restrict__ scale, int64_t n, CellGeom cell, double alpha, int64_t nlow,
                             int64_t nhigh, double inv_diel, double *__restrict__ gpos, double *__restrict__ partial) {
  __shared__ double red[8][7];
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = 0.0, v[6] = {0, 0, 0, 0, 0, 0};
  if (r < n) {
    int a = ab[r].x, b = ab[r].y;
    bool skip = (a < nlow && b < nlow) || (a >= nhigh && b >= nhigh);
    if (!skip) {
      double d[3] = {pos[3 * b] - pos[3 * a], pos[3 * b + 1] - pos[3 * a + 1], pos[3 * b + 2] - pos[3 * a + 2]};
      int m[3];
      exact_mic(d, cell, m);
      double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double x = alpha * dist;
      double pot = erf(x) / dist;
      double fac = (1.0 - scale[r]) * q[b] * q[a];
      double g = -fac * (1.1283791670955125739 * alpha * exp(-x * x) - pot) / dist / dist;
      e = -fac * pot * inv_diel;
      if (gpos) {
        for (int k = 0; k < 3; k++) {
          double y = d[k] * g * inv_diel;
          atomicAdd(gpos + 3 * b + k, y);
          atomicAdd(gpos + 3 * a + k, -y);
        }
      }
      g *= inv_diel;
      v[0] = d[0] * d[0] * g;
      v[1] = d[1] * d[1] * g;
      v[2] = d[2] * d[2] * g;
      v[3] = d[1] * d[0] * g;
      v[4] = d[2] * d[0] * g;
      v[5] = d[2] * d[1] * g;
    }
  }
  double vals[7] = {e, v[0], v[1], v[2], v[3], v[4], v[5]};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 7; k++) {
    double x = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    vals[k] = x;
  }
  if (lane == 0)
    for (int k = 0; k < 7; k++) red[wid][k] = vals[k];
  __syncthreads();
  if (threadIdx.x < 7) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 7 + threadIdx.x] = s;
  }
}

__global__ void k_store_corr_ev(const double *__restrict__ sums, double eself, double *__restrict__ ev) {
  if (threadIdx.x != 0) return;
  ev[0] = sums[0] + eself;
  double v[9] = {sums[1], sums[4], sums[5], sums[4], sums[2], sums[6], sums[5], sums[6], sums[3]};
  for (int q = 0; q < 9; q++) ev[1 + q] = v[q];
}

template <typename T> size_t force_smem(int nm, int RA) {
  size_t a = (size_t)nm * (16 * RA + EW_TC) * sizeof(typename C2<T>::t);
  size_t b = (size_t)16 * 16 * RA * 3 * sizeof(double);
  return a > b ? a : b;
}

template <typename T, typename TA, int RA>
int run_reci(yg_ctx *ctx, int want_grad) {
  typedef typename C2<T>::t CT;
  typedef typename C2<TA>::t CA;
  const int G0 = (int)ctx->ew_gmax[0], G1 = (int)ctx->ew_gmax[1], G2 = (int)ctx->ew_gmax[2];
  const int nm = G2 + 1;
  const int L = G0 + G1 + G2 + 3;
  const int64_t N = ctx->natom;
  const int ntile = ctx->ew_ntile;
  const int nmt = (nm + EW_MT - 1) / EW_MT;
  const int64_t nk_dense = (int64_t)ctx->ew_ncol * nm;
  int rc;
  // tables
  size_t tb = (size_t)N * L * sizeof(CT);
  if ((rc = yg_ensure(&ctx->d_ew_tab, &ctx->ew_bytes_tab, tb))) return rc;
  CT *tab = (CT *)ctx->d_ew_tab;
  k_tables<T><<<yg_blocks(N * L, 256), 256, 0, ctx->stream>>>(ctx->d_pos, ctx->d_charge, N, ctx->cell, G0, G1, G2, tab);
  YG_LAUNCH_CHECK(ctx, "k_tables");
  // atom groups: 0 = [nlow, nhigh) (always), 1 = [0, nlow), 2 = [nhigh, N)
  int64_t lo = ctx->ew_nlow, hi = ctx->ew_nhigh;
  int64_t gb[3][2] = {{lo, hi}, {0, lo}, {hi, N}};
  const int nS = (lo > 0 || hi < N) ? 3 : 1;
  // structure factors
  int maxchunk = 0;
  for (int g = 0; g < nS; g++) {
    int64_t n = gb[g][1] - gb[g][0];
    int nch = (int)((n + EW_ATB - 1) / EW_ATB);
    if (nch > maxchunk) maxchunk = nch;
  }
  if (maxchunk < 1) maxchunk = 1;
  size_t per = (size_t)ntile * nmt * EW_TC * EW_MT;
  if ((rc = yg_ensure(&ctx->d_ew_Spart, &ctx->ew_bytes_Spart, per * maxchunk * sizeof(CA)))) return rc;
  for (int g = 0; g < nS; g++) {
    int64_t n = gb[g][1] - gb[g][0];
    double *S = ctx->d_ew_S + (size_t)g * 2 * nk_dense;
    if (n <= 0) {
      YG_CUDA(cudaMemsetAsync(S, 0, 2 * nk_dense * sizeof(double), ctx->stream));
      continue;
    }
    int nch = (int)((n + EW_ATB - 1) / EW_ATB);
    dim3 grid(ntile, nch, nmt);
    YG_CUDA(cudaMemsetAsync(S, 0, 2 * nk_dense * sizeof(double), ctx->stream));
    k_sfac<T, TA><<<grid, 128, 0, ctx->stream>>>(tab, (int)gb[g][0], (int)gb[g][1], G0, G1, G2,
                                                 (const int4 *)ctx->d_ew_tiles, (CA *)ctx->d_ew_Spart, ntile);
    YG_LAUNCH_CHECK(ctx, "k_sfac");
    k_sfac_reduce<TA><<<yg_blocks((int64_t)per, 256), 256, 0, ctx->stream>>>(
        (const CA *)ctx->d_ew_Spart, nch, ntile, nmt, (const int4 *)ctx->d_ew_tiles, G0, G1, nm, S);
    YG_LAUNCH_CHECK(ctx, "k_sfac_reduce");
  }
  // energy, virial, weights
  const int ngroup = (nS == 3) ? 3 : 1;
  if ((rc = yg_ensure(&ctx->d_ew_W, &ctx->ew_bytes_W, (size_t)ngroup * nk_dense * sizeof(CT)))) return rc;
  const int eb = yg_blocks(nk_dense, 256);
  if ((rc = yg_ensure((void **)&ctx->d_red, &ctx->red_cap, ((size_t)eb * 7 + 64 + 7) * sizeof(double)))) return rc;
  double *partial = ctx->d_red + 64;
  const double fac2 = 0.25 / ctx->ew_alpha / ctx->ew_alpha;
  k_ewald_energy<T><<<eb, 256, 0, ctx->stream>>>(ctx->d_ew_S, nS, nk_dense, ctx->d_ew_pref, G0, G1, nm, ctx->cell,
                                                fac2, ngroup, (CT *)ctx->d_ew_W, partial);
  YG_LAUNCH_CHECK(ctx, "k_ewald_energy");
  double *sums = partial + (size_t)eb * 7;
  if ((rc = yg_launch_reduce_ev(ctx, partial, eb, 7, sums))) return rc;
  double *ev = ctx->d_part_ev + 10 * YG_PART_EWALD_RECI;
  k_store_ewald_ev<<<1, 32, 0, ctx->stream>>>(sums, 1.0 / ctx->ew_diel, ev);
  YG_LAUNCH_CHECK(ctx, "k_store_ewald_ev");
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_EWALD_RECI * N * 3;
  if (!want_grad) {
    YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_EWALD_RECI] = 1;
    return YG_OK;
  }
  // force pass, per atom group
  if ((rc = yg_ensure((void **)&ctx->d_ew_gpart, &ctx->ew_bytes_gpart, (size_t)N * 3 * sizeof(double)))) return rc;
  size_t smem = force_smem<T>(nm, RA);
  YG_CUDA(cudaFuncSetAttribute(k_ewald_force<T, RA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int gidx[3] = {0, 1, 2};
  for (int g = 0; g < nS; g++) {
    int64_t n = gb[g][1] - gb[g][0];
    if (n <= 0) continue;
    const CT *Wg = (const CT *)ctx->d_ew_W + (size_t)(ngroup == 1 ? 0 : gidx[g]) * nk_dense;
    int nblk = (int)((n + 16 * RA - 1) / (16 * RA));
    k_ewald_force<T, RA><<<nblk, 256, smem, ctx->stream>>>(tab, (int)gb[g][0], (int)gb[g][1], G0, G1, G2,
                                                          (const int4 *)ctx->d_ew_tiles, ntile, Wg, ctx->d_ew_gpart);
    YG_LAUNCH_CHECK(ctx, "k_ewald_force");
  }
  k_ewald_gpos<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(ctx->d_ew_gpart, N, ctx->cell,
                                                           -6.2831853071795864769 / ctx->ew_diel, gpos);
  YG_LAUNCH_CHECK(ctx, "k_ewald_gpos");
  ctx->part_valid[YG_PART_EWALD_RECI] = 1;
  return YG_OK;
}

}  // namespace

// Host-side k-space layout: prefactor grid in the reference's formula and
// the list of 8x8 column tiles that intersect the half sphere.
int yg_launch_ewald_setup(yg_ctx *ctx) {
  const int G0 = (int)ctx->ew_gmax[0], G1 = (int)ctx->ew_gmax[1], G2 = (int)ctx->ew_gmax[2];
  if (G2 + 1 > EW_MAXM) {
    yg_set_error("Ewald gmax[2] too large (G2+1 must be <= 64)");
    return YG_ERR_UNSUPPORTED;
  }
  const int nc0 = 2 * G0 + 1, nc1 = 2 * G1 + 1, nm = G2 + 1;
  const int64_t nk_dense = (int64_t)nc0 * nc1 * nm;
  std::vector<double> pref(nk_dense, 0.0);
  const double tp = 6.2831853071795864769, fp = 12.566370614359172954;
  double kv[9];
  for (int i = 0; i < 9; i++) kv[i] = tp * ctx->cell.gv[i];
  const double fac1 = fp / ctx->cell.volume;
  const double fac2 = 0.25 / ctx->ew_alpha / ctx->ew_alpha;
  double gc2 = ctx->ew_gcut * tp;
  gc2 *= gc2;
  int nk = 0;
  std::vector<int> colmhi(nc0 * nc1, -1);
  for (int g0 = -G0; g0 <= G0; g0++)
    for (int g1 = -G1; g1 <= G1; g1++)
      for (int g2 = 0; g2 <= G2; g2++) {
        if (g2 == 0) {
          if (g1 < 0) continue;
          if (g1 == 0 && g0 <= 0) continue;
        }
        double k[3];
        k[0] = (g0 * kv[0] + g1 * kv[3] + g2 * kv[6]);
        k[1] = (g0 * kv[1] + g1 * kv[4] + g2 * kv[7]);
        k[2] = (g0 * kv[2] + g1 * kv[5] + g2 * kv[8]);
        double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc2) continue;
        int64_t col = (int64_t)(g0 + G0) * nc1 + (g1 + G1);
        pref[col * nm + g2] = fac1 * std::exp(-ksq * fac2) / ksq;
        if (g2 > colmhi[col]) colmhi[col] = g2;
        nk++;
      }
  std::vector<int4> tiles;
  for (int b0 = -G0; b0 <= G0; b0 += 8)
    for (int b1 = -G1; b1 <= G1; b1 += 8) {
      int mhi = -1;
      for (int i0 = 0; i0 < 8; i0++)
        for (int i1 = 0; i1 < 8; i1++) {
          int g0 = b0 + i0, g1 = b1 + i1;
          if (g0 > G0 || g1 > G1) continue;
          int64_t col = (int64_t)(g0 + G0) * nc1 + (g1 + G1);
          mhi = std::max(mhi, colmhi[col]);
        }
      if (mhi >= 0) tiles.push_back(make_int4(b0, b1, mhi, 0));
    }
  ctx->ew_ncol = nc0 * nc1;
  ctx->ew_nm = nm;
  ctx->ew_nk = nk;
  ctx->ew_ntile = (int)tiles.size();
  cudaFree(ctx->d_ew_pref);
  cudaFree(ctx->d_ew_tiles);
  cudaFree(ctx->d_ew_S);
  ctx->d_ew_pref = nullptr;
  ctx->d_ew_tiles = nullptr;
  ctx->d_ew_S = nullptr;
  int rc;
  if ((rc = yg_alloc((void **)&ctx->d_ew_pref, nk_dense * sizeof(double)))) return rc;
  if ((rc = yg_alloc((void **)&ctx->d_ew_tiles, std::max<size_t>(1, tiles.size()) * sizeof(int4)))) return rc;
  if ((rc = yg_alloc((void **)&ctx->d_ew_S, 3 * 2 * nk_dense * sizeof(double)))) return rc;
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_pref, pref.data(), nk_dense * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  if (!tiles.empty())
    YG_CUDA(cudaMemcpyAsync(ctx->d_ew_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice,
                            ctx->stream));
  YG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->have_ewald = 1;
  return YG_OK;
}

int yg_launch_ewald_reci(yg_ctx *ctx, int want_grad) {
  if (ctx->ew_ntile == 0) {
    double *ev = ctx->d_part_ev + 10 * YG_PART_EWALD_RECI;
    YG_CUDA(cudaMemsetAsync(ev, 0, 10 * sizeof(double), ctx->stream));
    YG_CUDA(cudaMemsetAsync(ctx->d_part_gpos + (size_t)YG_PART_EWALD_RECI * ctx->natom * 3, 0,
                            ctx->natom * 3 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_EWALD_RECI] = 1;
    return YG_OK;
  }
  if (ctx->precision == YG_FP64) return run_reci<double, double, 2>(ctx, want_grad);
  return run_reci<float, float, 4>(ctx, want_grad);
}

int yg_launch_ewald_corr(yg_ctx *ctx, int want_grad) {
  const int64_t N = ctx->natom;
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_EWALD_CORR * N * 3;
  YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
  // self term on the host, in the reference's order (ewald.c:289-292)
  extern double yg_host_self_energy(yg_ctx * ctx);
  double eself = yg_host_self_energy(ctx);
  const int64_t n = ctx->nstab;
  const int nb = yg_blocks(n > 0 ? n : 1, 256);
  int rc;
  if ((rc = yg_ensure((void **)&ctx->d_red, &ctx->red_cap, ((size_t)nb * 7 + 64 + 7) * sizeof(double)))) return rc;
  double *partial = ctx->d_red + 64;
  k_ewald_corr<<<nb, 256, 0, ctx->stream>>>(ctx->d_pos, ctx->d_charge, ctx->d_stab_ab, ctx->d_stab_scale, n, ctx->cell,
                                            ctx->ew_alpha, ctx->ew_nlow, ctx->ew_nhigh, 1.0 / ctx->ew_diel,
                                            want_grad ? gpos : nullptr, partial);
  YG_LAUNCH_CHECK(ctx, "k_ewald_corr");
  double *sums = partial + (size_t)nb * 7;
  if ((rc = yg_launch_reduce_ev(ctx, partial, nb, 7, sums))) return rc;
  k_store_corr_ev<<<1, 32, 0, ctx->stream>>>(sums, eself / ctx->ew_diel, ctx->d_part_ev + 10 * YG_PART_EWALD_CORR);
  YG_LAUNCH_CHECK(ctx, "k_store_corr_ev");
  ctx->part_valid[YG_PART_EWALD_CORR] = 1;
  return YG_OK;
}
