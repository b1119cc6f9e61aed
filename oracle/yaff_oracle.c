/*
 * yaff_oracle.c -- CPU oracle for the force-evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke
 * entry and the CPU-baseline leg of bench.py call it to produce the expected
 * results; the product (yaff_gb300) never links or calls it.
 *
 * It restates, in plain C99 and in this project's own code, the algorithms of
 * the reference's native force-field core.  Every function keeps the
 * arithmetic order of the reference formula it restates (so the neighbour
 * pair set and the distances come out bit-identical when compiled with
 * -ffp-contract=off) and cites the reference file:line it follows.  Parity of
 * this restatement is pinned against the reference itself (built from its
 * sources by oracle/build_ref.sh) through the golden fixtures in
 * tests/golden/.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared yaff_oracle.c -lm
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

/* 2 pi, 4 pi, sqrt(pi), 2/sqrt(pi) to 20 significant digits */
#define ORC_TWO_PI 6.2831853071795864769
#define ORC_FOUR_PI 12.566370614359172954
#define ORC_SQRT_PI 1.7724538509055160273
#define ORC_TWO_DIV_SQRT_PI 1.1283791670955125739

/* Periodic cell: cell vectors as rows (rv) and reciprocal vectors as rows
 * (gv, gv = inv(rv)^T).  Mirrors the cell record of yaff/pes/cell.h:28-33. */
typedef struct {
  double rv[9];
  double gv[9];
  int nvec;
} orc_cell;

/* One neighbour-list row, same field layout as yaff/pes/nlist.h:30-35
 * (72 bytes: two int64 atom indices, distance, relative vector, image). */
typedef struct {
  int64_t a, b;
  double d, dx, dy, dz;
  int64_t r0, r1, r2;
} orc_neigh;

/* One exclusion/scaling row, layout of yaff/pes/pair_pot.h:46-50. */
typedef struct {
  int64_t a, b;
  double scale;
  int64_t nbond;
} orc_scale;

/* Relative-vector row, layout of yaff/pes/dlist.h:30-34. */
typedef struct {
  double dx, dy, dz;
  int64_t i, j;
  double gx, gy, gz;
} orc_delta;

/* Internal-coordinate row, layout of yaff/pes/iclist.h:30-38. */
typedef struct {
  int64_t kind;
  int64_t i0, sign0, i1, sign1, i2, sign2, i3, sign3;
  double value, grad;
} orc_ic;

/* Valence-term row, layout of yaff/pes/vlist.h:30-37. */
typedef struct {
  int64_t kind;
  double par0, par1, par2, par3, par4, par5;
  int64_t ic0, ic1;
  double energy;
} orc_vterm;

/* ---------------------------------------------------------------- cell -- */

/* Fractional wrap of a relative vector, one cell vector at a time; each
 * rounding sees the vector already wrapped along the previous axes.
 * Follows yaff/pes/cell.c:81-106 (cell_mic). */
static void orc_mic(double *d, const orc_cell *c) {
  int k;
  for (k = 0; k < c->nvec; k++) {
    const double *g = c->gv + 3 * k;
    const double *r = c->rv + 3 * k;
    double x = ceil(g[0] * d[0] + g[1] * d[1] + g[2] * d[2] - 0.5);
    d[0] -= x * r[0];
    d[1] -= x * r[1];
    d[2] -= x * r[2];
  }
}

/* Adds sum_k img[k]*rv[k] to d, axis by axis.  yaff/pes/cell.c:124-143. */
static void orc_add_vec(double *d, const orc_cell *c, const int64_t *img) {
  int k;
  for (k = 0; k < c->nvec; k++) {
    const double *r = c->rv + 3 * k;
    double m = (double)img[k];
    d[0] += m * r[0];
    d[1] += m * r[1];
    d[2] += m * r[2];
  }
}

/* Integer image that brings d into the central parallelepiped, all axes from
 * the same (unwrapped) d.  yaff/pes/cell.c:109-121 (cell_to_center). */
static void orc_to_center(const double *d, const orc_cell *c, int64_t *ctr) {
  int k;
  for (k = 0; k < c->nvec; k++) {
    const double *g = c->gv + 3 * k;
    ctr[k] = (int64_t)(-ceil(g[0] * d[0] + g[1] * d[1] + g[2] * d[2] - 0.5));
  }
}

void orc_mic_vec(double *d, const double *rv, const double *gv, int nvec) {
  orc_cell c;
  int i;
  for (i = 0; i < 9; i++) { c.rv[i] = rv[i]; c.gv[i] = gv[i]; }
  c.nvec = nvec;
  orc_mic(d, &c);
}

/* --------------------------------------------------------------- nlist -- */

/* Advance the image counter over the half space of images (central image
 * first, then r0 fastest); returns 0 and resets to the central image when
 * all images were visited.  yaff/pes/nlist.c:137-180 (nlist_inc_r). */
static int orc_next_image(const orc_cell *c, int64_t *r, const int64_t *rmax) {
  int k;
  if (c->nvec == 0) return 0;
  for (k = 0; k < c->nvec; k++) {
    r[k]++;
    if (r[k] <= rmax[k]) return 1;
    r[k] = -rmax[k];
  }
  for (k = 0; k < c->nvec; k++) r[k] = 0;
  return 0;
}

/* Full rebuild of the half neighbour list: all (a, b, image) with
 * |MIC(pos[b]-pos[a]) +/- image| < rcut over the half space of images,
 * rows ordered exactly as the reference produces them.  Writes at most `cap`
 * rows; returns the total number of rows (callers regrow and rerun when the
 * total exceeds `cap`).  yaff/pes/nlist.c:30-131 (nlist_build_low) with the
 * status protocol of yaff/pes/nlist.py:163-186 replaced by count-and-retry. */
int64_t orc_nlist_build_range(const double *pos, int64_t natom, double rcut,
                              const int64_t *rmax, const double *rv, const double *gv,
                              int nvec, int64_t nlow, int64_t nhigh, int64_t a_begin,
                              int64_t a_end, orc_neigh *out, int64_t cap);

int64_t orc_nlist_build(const double *pos, int64_t natom, double rcut,
                        const int64_t *rmax, const double *rv, const double *gv,
                        int nvec, int64_t nlow, int64_t nhigh,
                        orc_neigh *out, int64_t cap) {
  return orc_nlist_build_range(pos, natom, rcut, rmax, rv, gv, nvec, nlow, nhigh, nlow, natom, out, cap);
}

/* The rows of orc_nlist_build whose first loop index a lies in
 * [a_begin, a_end), in the same order (the full list is the concatenation of
 * consecutive ranges). */
int64_t orc_nlist_build_range(const double *pos, int64_t natom, double rcut,
                              const int64_t *rmax, const double *rv, const double *gv,
                              int nvec, int64_t nlow, int64_t nhigh, int64_t a_begin,
                              int64_t a_end, orc_neigh *out, int64_t cap) {
  orc_cell c;
  int64_t a, b, n = 0, k;
  double rc2 = rcut * rcut;
  (void)natom;
  for (k = 0; k < 9; k++) { c.rv[k] = rv[k]; c.gv[k] = gv[k]; }
  c.nvec = nvec;
  for (a = a_begin; a < a_end; a++) {
    for (b = 0; b <= a; b++) {
      double d0[3];
      int64_t r[3] = {0, 0, 0};
      int image = 0;
      if (!((a >= nlow && b < nhigh) || (b >= nlow && a < nhigh))) continue;
      d0[0] = pos[3 * b] - pos[3 * a];
      d0[1] = pos[3 * b + 1] - pos[3 * a + 1];
      d0[2] = pos[3 * b + 2] - pos[3 * a + 2];
      orc_mic(d0, &c);
      for (;;) {
        int nsign = (image && a != b) ? 2 : 1;
        int s;
        if (b < a || image) {
          for (s = 0; s < nsign; s++) {
            double sign = (s == 0) ? 1.0 : -1.0;
            double d[3], dd;
            d[0] = sign * d0[0];
            d[1] = sign * d0[1];
            d[2] = sign * d0[2];
            orc_add_vec(d, &c, r);
            dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (dd < rc2) {
              if (n < cap) {
                orc_neigh *row = out + n;
                row->a = (s == 0) ? a : b;
                row->b = (s == 0) ? b : a;
                row->d = sqrt(dd);
                row->dx = d[0];
                row->dy = d[1];
                row->dz = d[2];
                row->r0 = r[0];
                row->r1 = r[1];
                row->r2 = r[2];
              }
              n++;
            }
          }
        }
        if (!orc_next_image(&c, r, rmax)) break;
        image = 1;
      }
    }
  }
  return n;
}

/* Skin path: keep the rows, recompute relative vectors from the new positions
 * with the image that brought the old relative vector to the centre.
 * yaff/pes/nlist.c:183-232 (nlist_recompute_low). */
void orc_nlist_recompute(const double *pos, const double *pos_old,
                         const double *rv, const double *gv, int nvec,
                         orc_neigh *rows, int64_t n) {
  orc_cell c;
  int64_t i, k, a = -1, b = -1;
  double d0[3] = {0, 0, 0};
  for (k = 0; k < 9; k++) { c.rv[k] = rv[k]; c.gv[k] = gv[k]; }
  c.nvec = nvec;
  for (i = 0; i < n; i++) {
    orc_neigh *row = rows + i;
    double d[3];
    int64_t img[3];
    if (row->a != a || row->b != b) {
      int64_t ctr[3] = {0, 0, 0};
      a = row->a;
      b = row->b;
      d0[0] = pos_old[3 * b] - pos_old[3 * a];
      d0[1] = pos_old[3 * b + 1] - pos_old[3 * a + 1];
      d0[2] = pos_old[3 * b + 2] - pos_old[3 * a + 2];
      orc_to_center(d0, &c, ctr);
      d0[0] = pos[3 * b] - pos[3 * a];
      d0[1] = pos[3 * b + 1] - pos[3 * a + 1];
      d0[2] = pos[3 * b + 2] - pos[3 * a + 2];
      orc_add_vec(d0, &c, ctr);
    }
    d[0] = d0[0];
    d[1] = d0[1];
    d[2] = d0[2];
    img[0] = row->r0;
    img[1] = row->r1;
    img[2] = row->r2;
    orc_add_vec(d, &c, img);
    row->d = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    row->dx = d[0];
    row->dy = d[1];
    row->dz = d[2];
  }
}

/* --------------------------------------------------------- pair terms -- */

enum { ORC_LJ = 0, ORC_MM3 = 1, ORC_EI = 2, ORC_MM3CAP = 3, ORC_GRIMME = 4, ORC_EXPREP = 5, ORC_QMDFFREP = 6,
       ORC_LJCROSS = 7, ORC_DAMPDISP = 8, ORC_DISP68BJ = 9 };
enum { ORC_TR_NONE = 0, ORC_TR_HAMMER = 1, ORC_TR_SWITCH3 = 2 };

typedef struct {
  int kind;
  const double *sigma, *epsilon;   /* LJ, MM3, MM3CAP; Grimme: r0, c6 */
  const int32_t *onlypauli;        /* MM3, MM3CAP */
  const double *charges, *radii;   /* EI */
  double alpha, dielectric;        /* EI */
  const int64_t *types;            /* type-pair table kinds */
  int64_t ntype, power;
  const double *cross0, *cross1, *cross2;
  double c6_scale, c8_scale, bj_a, bj_b;
  double rcut;
  int tr_kind;
  double tr_par;
} orc_pairpot;

/* Hammer truncation exp(tau/(d-rcut)).  yaff/pes/truncation.c:30-41. */
static double orc_hammer(double d, double rcut, double tau, double *g) {
  if (d < rcut) {
    double x = d - rcut;
    double h = exp(tau / x);
    if (g) *g = -h * tau / x / x;
    return h;
  }
  if (g) *g = 0.0;
  return 0.0;
}

/* Cubic switching over [rcut-width, rcut].  yaff/pes/truncation.c:59-76. */
static double orc_switch3(double d, double rcut, double width, double *g) {
  if (d < rcut) {
    double x = rcut - d;
    if (x > width) {
      if (g) *g = 0.0;
      return 1.0;
    }
    x /= width;
    if (g) *g = -6 * x * (1 - x) / width;
    return (3 - 2 * x) * x * x;
  }
  if (g) *g = 0.0;
  return 0.0;
}

/* Lennard-Jones 4 eps (x^2 - x), x = (sigma/d)^6, arithmetic-mean sigma and
 * geometric-mean epsilon.  yaff/pes/pair_pot.c:277-301 (pair_fn_lj). */
static double orc_lj(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  double sig = 0.5 * (p->sigma[i] + p->sigma[j]);
  double eps = sqrt(p->epsilon[i] * p->epsilon[j]);
  double x = sig / d;
  x *= x;
  x *= x * x;
  if (g) *g = 24.0 * eps / d / d * x * (1.0 - 2.0 * x);
  return 4.0 * eps * (x * (x - 1.0));
}

/* MM3 exp-6: eps (1.84e5 exp(-12 d/sigma) - 2.25 (sigma/d)^6) with
 * sigma = sigma_i + sigma_j (a sum, not a mean) and an only-Pauli switch.
 * yaff/pes/pair_pot.c:321-352 (pair_fn_mm3). */
static double orc_mm3(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  double sig = p->sigma[i] + p->sigma[j];
  double eps = sqrt(p->epsilon[i] * p->epsilon[j]);
  int op = p->onlypauli[i] + p->onlypauli[j];
  double x = sig / d;
  double ex = 1.84e5 * exp(-12.0 / x);
  if (op == 0) {
    x *= x;
    x *= 2.25 * x * x;
    if (g) *g = eps / d * (-12.0 / sig * ex + 6.0 / d * x);
    return eps * (ex - x);
  }
  if (g) *g = eps / d * (-12.0 / sig * ex);
  return eps * ex;
}

/* Real-space Ewald / Coulomb term between point or Gaussian charges.
 * yaff/pes/pair_pot.c:711-751 (pair_fn_ei). */
static double orc_ei(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  double qq = (p->charges[i] * p->charges[j]) / p->dielectric;
  double rij = 0.0, pot, x, y;
  if (p->radii) rij = sqrt(p->radii[i] * p->radii[i] + p->radii[j] * p->radii[j]);
  if (p->alpha > 0) {
    x = p->alpha * d;
    if (rij > 0) {
      y = d / rij;
      pot = qq / d * (erfc(x) - erfc(y));
      if (g) *g = (ORC_TWO_DIV_SQRT_PI * (exp(-y * y) / rij - exp(-x * x) * p->alpha) * qq - pot) / (d * d);
    } else {
      pot = qq * erfc(x) / d;
      if (g) *g = (-ORC_TWO_DIV_SQRT_PI * p->alpha * exp(-x * x) * qq - pot) / (d * d);
    }
  } else {
    if (rij > 0) {
      y = d / rij;
      pot = qq / d * erf(y);
      if (g) *g = (ORC_TWO_DIV_SQRT_PI / rij * exp(-y * y) * qq - pot) / (d * d);
    } else {
      pot = qq / d;
      if (g) *g = -pot / (d * d);
    }
  }
  return pot;
}

/* MM3 with a linear cap below x = d/sigma = 0.355114; below the cap the
 * gradient is the unmodified MM3 expression evaluated at the cap's x (so it
 * is not the derivative of the capped energy).  yaff/pes/pair_pot.c:373-419
 * (pair_fn_mm3cap). */
static double orc_mm3cap(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  double sig = p->sigma[i] + p->sigma[j];
  double eps = sqrt(p->epsilon[i] * p->epsilon[j]);
  int op = p->onlypauli[i] + p->onlypauli[j];
  double x = d / sig, xmax = 0.355114, ex;
  if (op != 0) return orc_mm3(p, i, j, d, g);
  if (x > xmax) {
    ex = 1.84e5 * exp(-12.0 * x);
    x *= x;
    x *= 1 / 2.25 * x * x;
    if (g) *g = eps / d * (-12.0 / sig * ex + 6.0 / d / x);
    return eps * (ex - 1 / x);
  }
  ex = 1.84e5 * exp(-12.0 * xmax);
  xmax *= xmax;
  xmax *= 1 / 2.25 * xmax * xmax;
  if (g) *g = eps / d * (-12.0 / sig * ex + 6.0 / d / xmax);
  return eps * (5799.303156 - 12182.86986 * x);
}

/* Damped dispersion -1.1 f c6/d^6, f = 1/(1 + exp(-20 (d/r0 - 1))), r0 the
 * sum and c6 the geometric mean.  yaff/pes/pair_pot.c:434-455. */
static double orc_grimme(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  double r0 = p->sigma[i] + p->sigma[j];
  double c6 = sqrt(p->epsilon[i] * p->epsilon[j]);
  double ex = exp(-20.0 * (d / r0 - 1.0));
  double f = 1.0 / (1.0 + ex);
  double d6 = d * d * d, e;
  d6 *= d6;
  e = 1.1 * f * c6 / d6;
  if (g) *g = e / d * (6.0 / d - 20.0 / r0 * f * ex);
  return -e;
}

static int64_t orc_tpair(const orc_pairpot *p, int64_t i, int64_t j) {
  return p->types[i] * p->ntype + p->types[j];
}

/* A exp(-B d) (ExpRep) and A exp(-B d)/d (QMDFFRep) per type pair; zero
 * when A or B is zero.  yaff/pes/pair_pot.c:473-489, :506-522. */
static double orc_rep(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  int64_t k = orc_tpair(p, i, j);
  double amp = p->cross0[k], b = p->cross1[k], e;
  if (amp == 0.0 || b == 0.0) {
    if (g) *g = 0.0;
    return 0.0;
  }
  if (p->kind == ORC_EXPREP) {
    e = amp * exp(-b * d);
    if (g) *g = -e * b / d;
  } else {
    e = amp / d * exp(-b * d);
    if (g) *g = -(b + 1 / d) * e / d;
  }
  return e;
}

/* Lennard-Jones with per-type-pair epsilon and sigma.
 * yaff/pes/pair_pot.c:540-557. */
static double orc_ljcross(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  int64_t k = orc_tpair(p, i, j);
  double eps = p->cross0[k], sig = p->cross1[k], x = sig / d;
  x *= x;
  x *= x * x;
  if (g) *g = 24.0 * eps / d / d * x * (1.0 - 2.0 * x);
  return 4.0 * eps * (x * (x - 1.0));
}

/* Tang-Toennies damping 1 - exp(-x) sum_{k=0..n} x^k/k!; *g = exp(-x)
 * x^n/n!.  yaff/pes/pair_pot.c:576-594. */
static double orc_tang_toennies(double x, int order, double *g) {
  double tmp = 1.0, poly = 0.0, last, e;
  int k, fac = 1;
  for (k = 0; k < order; k++) {
    poly += tmp / fac;
    fac *= k + 1;
    tmp *= x;
  }
  last = tmp / fac;
  poly += last;
  e = exp(-x);
  if (g) *g = e * last;
  return 1.0 - poly * e;
}

/* -C/d^n, Tang-Toennies damped where B != 0.  yaff/pes/pair_pot.c:596-629. */
static double orc_dampdisp(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  int64_t k = orc_tpair(p, i, j), q;
  double cn = p->cross0[k], b = p->cross1[k], disp = 1.0, damp;
  if (cn == 0.0) return 0.0;
  for (q = 0; q < p->power; q++) disp *= d;
  disp = -cn / disp;
  if (b == 0.0) {
    if (g) *g = -p->power * disp / (d * d);
    return disp;
  }
  damp = orc_tang_toennies(b * d, (int)p->power, g);
  if (g) *g = ((*g) * b - p->power / d * damp) * disp / d;
  return damp * disp;
}

/* Becke-Johnson damped C6 + C8 dispersion, R = bj_a R_ij + bj_b.
 * yaff/pes/pair_pot.c:651-677. */
static double orc_disp68bj(const orc_pairpot *p, int64_t i, int64_t j, double d, double *g) {
  int64_t k = orc_tpair(p, i, j);
  double c6 = p->cross0[k], c8 = p->cross1[k];
  double R = p->bj_a * p->cross2[k] + p->bj_b;
  double R2 = R * R, R4 = R2 * R2, R6 = R4 * R2, R8 = R4 * R4;
  double d2 = d * d, d4 = d2 * d2, d6 = d4 * d2, d8 = d4 * d4;
  double pot = -p->c6_scale * c6 / (d6 + R6) - p->c8_scale * c8 / (d8 + R8);
  if (g) *g = 6.0 * p->c6_scale * c6 / (d6 + R6) / (d6 + R6) * d4 + 8.0 * p->c8_scale * c8 / (d8 + R8) / (d8 + R8) * d6;
  return pot;
}

/* Scaling factor of pair (a, b) from the (a, b)-sorted table, walked in lock
 * step with the (a, b)-sorted neighbour list.  yaff/pes/pair_pot.c:65-81. */
static double orc_get_scaling(const orc_scale *st, int64_t a, int64_t b, int64_t *row, int64_t n) {
  if (*row >= n) return 1.0;
  while (st[*row].a < a) {
    (*row)++;
    if (*row >= n) return 1.0;
  }
  if (st[*row].a != a) return 1.0;
  while (st[*row].b < b) {
    (*row)++;
    if (*row >= n) return 1.0;
    if (st[*row].a != a) return 1.0;
  }
  if (st[*row].b == b && st[*row].a == a) return st[*row].scale;
  return 1.0;
}

typedef double (*orc_pair_fn)(const orc_pairpot *, int64_t, int64_t, double, double *);

static orc_pair_fn orc_pair_fn_of(int kind) {
  switch (kind) {
    case ORC_LJ: return orc_lj;
    case ORC_MM3: return orc_mm3;
    case ORC_EI: return orc_ei;
    case ORC_MM3CAP: return orc_mm3cap;
    case ORC_GRIMME: return orc_grimme;
    case ORC_EXPREP: case ORC_QMDFFREP: return orc_rep;
    case ORC_LJCROSS: return orc_ljcross;
    case ORC_DAMPDISP: return orc_dampdisp;
    case ORC_DISP68BJ: return orc_disp68bj;
    default: return 0;
  }
}

static double orc_pair_loop(const orc_neigh *rows, int64_t n, const orc_scale *st, int64_t nst,
                            const orc_pairpot *pp, double *gpos, double *vtens);

/* Generic pair loop with exclusion scaling, truncation chain rule, gradient
 * and virial accumulation.  yaff/pes/pair_pot.c:84-176 (pair_pot_compute). */
double orc_pair_compute(const orc_neigh *rows, int64_t n, const orc_scale *st,
                        int64_t nst, int kind, const double *sigma,
                        const double *epsilon, const int32_t *onlypauli,
                        const double *charges, const double *radii,
                        double alpha, double dielectric, double rcut,
                        int tr_kind, double tr_par, double *gpos, double *vtens) {
  orc_pairpot p = {0};
  p.kind = kind; p.sigma = sigma; p.epsilon = epsilon; p.onlypauli = onlypauli;
  p.charges = charges; p.radii = radii; p.alpha = alpha; p.dielectric = dielectric;
  p.rcut = rcut; p.tr_kind = tr_kind; p.tr_par = tr_par;
  return orc_pair_loop(rows, n, st, nst, &p, gpos, vtens);
}

/* The same loop for the type-pair table kinds (ExpRep, QMDFFRep, LJCross,
 * DampDisp, Disp68BJDamp); tables are ntype x ntype row-major, scales =
 * {c6_scale, c8_scale, bj_a, bj_b} or NULL. */
double orc_pair_compute_table(const orc_neigh *rows, int64_t n, const orc_scale *st, int64_t nst, int kind,
                              const int64_t *types, int64_t ntype, const double *cross0, const double *cross1,
                              const double *cross2, int64_t power, const double *scales, double rcut,
                              int tr_kind, double tr_par, double *gpos, double *vtens) {
  orc_pairpot p = {0};
  p.kind = kind; p.types = types; p.ntype = ntype; p.power = power;
  p.cross0 = cross0; p.cross1 = cross1; p.cross2 = cross2;
  if (scales) { p.c6_scale = scales[0]; p.c8_scale = scales[1]; p.bj_a = scales[2]; p.bj_b = scales[3]; }
  p.rcut = rcut; p.tr_kind = tr_kind; p.tr_par = tr_par;
  return orc_pair_loop(rows, n, st, nst, &p, gpos, vtens);
}

static double orc_pair_loop(const orc_neigh *rows, int64_t n, const orc_scale *st, int64_t nst,
                            const orc_pairpot *pp, double *gpos, double *vtens) {
  const orc_pairpot *p = pp;
  orc_pair_fn fn = orc_pair_fn_of(p->kind);
  const int tr_kind = p->tr_kind;
  const double rcut = p->rcut, tr_par = p->tr_par;
  int64_t i, srow = 0;
  double energy = 0.0;
  if (!fn) return NAN;
  for (i = 0; i < n; i++) {
    const orc_neigh *r = rows + i;
    double s, v, vg = 0.0, h, hg;
    int want_g = (gpos != NULL) || (vtens != NULL);
    if (!(r->d < rcut)) continue;
    if (r->r0 == 0 && r->r1 == 0 && r->r2 == 0)
      s = orc_get_scaling(st, r->a, r->b, &srow, nst);
    else
      s = 1.0;
    if (s == 0.0) continue;
    v = fn(p, r->a, r->b, r->d, want_g ? &vg : NULL);
    if (!want_g) {
      if (tr_kind != ORC_TR_NONE && v != 0.0) {
        v *= (tr_kind == ORC_TR_HAMMER) ? orc_hammer(r->d, rcut, tr_par, NULL)
                                        : orc_switch3(r->d, rcut, tr_par, NULL);
      }
    } else {
      if (tr_kind != ORC_TR_NONE && (v != 0.0 || vg != 0.0)) {
        h = (tr_kind == ORC_TR_HAMMER) ? orc_hammer(r->d, rcut, tr_par, &hg)
                                       : orc_switch3(r->d, rcut, tr_par, &hg);
        vg = vg * h + v * hg / r->d;
        v *= h;
      }
      vg *= s;
      if (gpos) {
        h = r->dx * vg;
        gpos[3 * r->b] += h;
        gpos[3 * r->a] -= h;
        h = r->dy * vg;
        gpos[3 * r->b + 1] += h;
        gpos[3 * r->a + 1] -= h;
        h = r->dz * vg;
        gpos[3 * r->b + 2] += h;
        gpos[3 * r->a + 2] -= h;
      }
      if (vtens) {
        vtens[0] += r->dx * (r->dx * vg);
        vtens[4] += r->dy * (r->dy * vg);
        vtens[8] += r->dz * (r->dz * vg);
        vtens[1] += r->dx * (r->dy * vg);
        vtens[3] += r->dy * (r->dx * vg);
        vtens[2] += r->dx * (r->dz * vg);
        vtens[6] += r->dz * (r->dx * vg);
        vtens[5] += r->dy * (r->dz * vg);
        vtens[7] += r->dz * (r->dy * vg);
      }
    }
    energy += s * v;
  }
  return energy;
}

/* ---------------------------------------------------------------- Ewald -- */

/* Direct reciprocal-space sum over the half sphere |k| <= 2 pi gcut, with
 * the nlow/nhigh split (E = S0 (S0 + 2 (S1+S2)) + 2 S1 S2).
 * yaff/pes/ewald.c:32-150 (compute_ewald_reci). */
double orc_ewald_reci_range(const double *pos, int64_t natom, int64_t nlow, int64_t nhigh,
                            const double *charges, const double *gv, double volume, double alpha,
                            const int64_t *gmax, double gcut, int64_t k_begin, int64_t k_end,
                            double *gpos, double *work, double *vtens);

double orc_ewald_reci(const double *pos, int64_t natom, int64_t nlow, int64_t nhigh,
                      const double *charges, const double *rv, const double *gv,
                      double volume, double alpha, const int64_t *gmax,
                      double gcut, double dielectric, double *gpos,
                      double *work, double *vtens) {
  double energy, dfac;
  int64_t i;
  (void)rv;
  energy = orc_ewald_reci_range(pos, natom, nlow, nhigh, charges, gv, volume, alpha, gmax, gcut, 0, INT64_MAX,
                                gpos, work, vtens);
  if (vtens) { vtens[0] -= energy; vtens[4] -= energy; vtens[8] -= energy; }
  dfac = 1.0 / dielectric;
  if (gpos) for (i = 0; i < 3 * natom; i++) gpos[i] *= dfac;
  if (vtens) for (i = 0; i < 9; i++) vtens[i] *= dfac;
  return energy * dfac;
}

/* The k-vectors of orc_ewald_reci with index (in the loop order of the half
 * sphere, counting only those inside the cutoff) in [k_begin, k_end): their
 * energy sum, with their gradient and virial terms added to gpos / vtens,
 * before the dielectric scaling and the -E diagonal of the virial. */
double orc_ewald_reci_range(const double *pos, int64_t natom, int64_t nlow, int64_t nhigh,
                            const double *charges, const double *gv, double volume, double alpha,
                            const int64_t *gmax, double gcut, int64_t k_begin, int64_t k_end,
                            double *gpos, double *work, double *vtens) {
  double kv[9], energy = 0.0, fac1, fac2, gc2;
  int64_t g0, g1, g2, i, kidx = -1;
  for (i = 0; i < 9; i++) kv[i] = ORC_TWO_PI * gv[i];
  fac1 = ORC_FOUR_PI / volume;
  fac2 = 0.25 / alpha / alpha;
  gc2 = gcut * ORC_TWO_PI;
  gc2 *= gc2;
  for (g0 = -gmax[0]; g0 <= gmax[0]; g0++) {
    for (g1 = -gmax[1]; g1 <= gmax[1]; g1++) {
      for (g2 = 0; g2 <= gmax[2]; g2++) {
        double k[3], ksq, cm = 0, sm = 0, cl = 0, sl = 0, ch = 0, sh = 0, c, s, x;
        if (g2 == 0) {
          if (g1 < 0) continue;
          if (g1 == 0 && g0 <= 0) continue;
        }
        k[0] = (g0 * kv[0] + g1 * kv[3] + g2 * kv[6]);
        k[1] = (g0 * kv[1] + g1 * kv[4] + g2 * kv[7]);
        k[2] = (g0 * kv[2] + g1 * kv[5] + g2 * kv[8]);
        ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc2) continue;
        kidx++;
        if (kidx < k_begin) continue;
        if (kidx >= k_end) return energy;
        for (i = 0; i < natom; i++) {
          x = k[0] * pos[3 * i] + k[1] * pos[3 * i + 1] + k[2] * pos[3 * i + 2];
          c = charges[i] * cos(x);
          s = charges[i] * sin(x);
          if (i < nlow) { cl += c; sl += s; }
          else if (i >= nhigh) { ch += c; sh += s; }
          else { cm += c; sm += s; }
          if (gpos) { work[2 * i] = c; work[2 * i + 1] = -s; }
        }
        c = fac1 * exp(-ksq * fac2) / ksq;
        s = cm * (cm + 2.0 * (cl + ch)) + sm * (sm + 2.0 * (sl + sh));
        s += 2.0 * (cl * ch + sl * sh);
        energy += c * s;
        if (gpos) {
          x = 2.0 * c;
          cm *= x; sm *= x; cl *= x; sl *= x; ch *= x; sh *= x;
          for (i = 0; i < natom; i++) {
            x = cm * work[2 * i + 1] + sm * work[2 * i];
            if (i < nhigh) x += ch * work[2 * i + 1] + sh * work[2 * i];
            if (i >= nlow) x += cl * work[2 * i + 1] + sl * work[2 * i];
            gpos[3 * i] += k[0] * x;
            gpos[3 * i + 1] += k[1] * x;
            gpos[3 * i + 2] += k[2] * x;
          }
        }
        if (vtens) {
          c *= 2.0 * (1.0 / ksq + fac2) * s;
          vtens[0] += c * k[0] * k[0];
          vtens[4] += c * k[1] * k[1];
          vtens[8] += c * k[2] * k[2];
          x = c * k[1] * k[0]; vtens[1] += x; vtens[3] += x;
          x = c * k[2] * k[0]; vtens[2] += x; vtens[6] += x;
          x = c * k[2] * k[1]; vtens[5] += x; vtens[7] += x;
        }
      }
    }
  }
  return energy;
}

/* Ewald self-energy and the reciprocal-space double counting of scaled
 * (excluded) pairs.  yaff/pes/ewald.c:278-349 (compute_ewald_corr). */
double orc_ewald_corr(const double *pos, const double *charges, const double *rv,
                      const double *gv, int nvec, double alpha,
                      const orc_scale *st, int64_t nst, double dielectric,
                      double *gpos, double *vtens, int64_t natom, int64_t nlow,
                      int64_t nhigh) {
  orc_cell c;
  int64_t i, k;
  double energy = 0.0, x, dfac;
  for (k = 0; k < 9; k++) { c.rv[k] = rv[k]; c.gv[k] = gv[k]; }
  c.nvec = nvec;
  x = alpha / ORC_SQRT_PI;
  for (i = nlow; i < nhigh; i++) energy -= x * charges[i] * charges[i];
  for (i = 0; i < nst; i++) {
    int64_t a = st[i].a, b = st[i].b;
    double d[3], dist, pot, fac, g = 0.0, y;
    if (a < nlow && b < nlow) continue;
    if (a >= nhigh && b >= nhigh) continue;
    d[0] = pos[3 * b] - pos[3 * a];
    d[1] = pos[3 * b + 1] - pos[3 * a + 1];
    d[2] = pos[3 * b + 2] - pos[3 * a + 2];
    orc_mic(d, &c);
    dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    y = alpha * dist;
    pot = erf(y) / dist;
    fac = (1 - st[i].scale) * charges[b] * charges[a];
    if (gpos || vtens) g = -fac * (ORC_TWO_DIV_SQRT_PI * alpha * exp(-y * y) - pot) / dist / dist;
    if (gpos) {
      y = d[0] * g; gpos[3 * b] += y; gpos[3 * a] -= y;
      y = d[1] * g; gpos[3 * b + 1] += y; gpos[3 * a + 1] -= y;
      y = d[2] * g; gpos[3 * b + 2] += y; gpos[3 * a + 2] -= y;
    }
    if (vtens) {
      vtens[0] += d[0] * d[0] * g;
      vtens[4] += d[1] * d[1] * g;
      vtens[8] += d[2] * d[2] * g;
      y = d[1] * d[0] * g; vtens[1] += y; vtens[3] += y;
      y = d[2] * d[0] * g; vtens[2] += y; vtens[6] += y;
      y = d[2] * d[1] * g; vtens[5] += y; vtens[7] += y;
    }
    energy -= fac * pot;
  }
  dfac = 1.0 / dielectric;
  if (gpos) for (i = 0; i < 3 * natom; i++) gpos[i] *= dfac;
  if (vtens) for (i = 0; i < 9; i++) vtens[i] *= dfac;
  return energy * dfac;
}

/* Reciprocal prefactors on the (2gmax0+1, 2gmax1+1, gmax2+1) grid with the
 * 1-based index shift of the reference.  yaff/pes/ewald.c:441-471. */
void orc_ewald_prefactors(const double *gv, double volume, double alpha,
                          const int64_t *gmax, double gcut, double *pref) {
  double kv[9], fac1, fac2, gc2;
  int64_t g0, g1, g2, i, idx = 0;
  for (i = 0; i < 9; i++) kv[i] = ORC_TWO_PI * gv[i];
  fac1 = ORC_FOUR_PI / volume;
  fac2 = 0.25 / alpha / alpha;
  gc2 = gcut * ORC_TWO_PI;
  gc2 *= gc2;
  for (g0 = -gmax[0]; g0 <= gmax[0]; g0++)
    for (g1 = -gmax[1]; g1 <= gmax[1]; g1++)
      for (g2 = 0; g2 <= gmax[2]; g2++) {
        double k[3], ksq;
        idx++;
        if (g2 == 0) {
          if (g1 < 0) continue;
          if (g1 == 0 && g0 <= 0) continue;
        }
        k[0] = (g0 * kv[0] + g1 * kv[3] + g2 * kv[6]);
        k[1] = (g0 * kv[1] + g1 * kv[4] + g2 * kv[7]);
        k[2] = (g0 * kv[2] + g1 * kv[5] + g2 * kv[8]);
        ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc2) continue;
        pref[idx] = fac1 * exp(-ksq * fac2) / ksq;
      }
}

/* Structure factors of a set of charges on the same grid (accumulated).
 * yaff/pes/ewald.c:473-506. */
void orc_ewald_structurefactors(const double *pos, int64_t natom,
                                const double *charges, const double *gv,
                                const int64_t *gmax, double gcut,
                                double *cosfacs, double *sinfacs) {
  double kv[9], gc2;
  int64_t g0, g1, g2, i, idx = 0;
  for (i = 0; i < 9; i++) kv[i] = ORC_TWO_PI * gv[i];
  gc2 = gcut * ORC_TWO_PI;
  gc2 *= gc2;
  for (g0 = -gmax[0]; g0 <= gmax[0]; g0++)
    for (g1 = -gmax[1]; g1 <= gmax[1]; g1++)
      for (g2 = 0; g2 <= gmax[2]; g2++) {
        double k[3], ksq;
        idx++;
        if (g2 == 0) {
          if (g1 < 0) continue;
          if (g1 == 0 && g0 <= 0) continue;
        }
        k[0] = (g0 * kv[0] + g1 * kv[3] + g2 * kv[6]);
        k[1] = (g0 * kv[1] + g1 * kv[4] + g2 * kv[7]);
        k[2] = (g0 * kv[2] + g1 * kv[5] + g2 * kv[8]);
        ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc2) continue;
        for (i = 0; i < natom; i++) {
          double x = k[0] * pos[3 * i] + k[1] * pos[3 * i + 1] + k[2] * pos[3 * i + 2];
          cosfacs[idx] += charges[i] * cos(x);
          sinfacs[idx] += charges[i] * sin(x);
        }
      }
}

/* Energy change from a structure-factor change.  yaff/pes/ewald.c:508-522. */
double orc_ewald_deltae(const double *dcos, const double *cosf, const double *dsin,
                        const double *sinf, const double *pref, int64_t nk) {
  int64_t i;
  double e = 0.0;
  for (i = 0; i < nk; i++) e += (cosf[i] * dcos[i] + sinf[i] * dsin[i]) * pref[i];
  return 2.0 * e;
}

/* ------------------------------------------------------------- valence -- */

/* Layer 1 forward: MIC relative vectors.  yaff/pes/dlist.c:29-42. */
void orc_dlist_forward(const double *pos, const double *rv, const double *gv,
                       int nvec, orc_delta *dl, int64_t n) {
  orc_cell c;
  int64_t k;
  for (k = 0; k < 9; k++) { c.rv[k] = rv[k]; c.gv[k] = gv[k]; }
  c.nvec = nvec;
  for (k = 0; k < n; k++) {
    orc_delta *r = dl + k;
    double d[3];
    d[0] = pos[3 * r->j] - pos[3 * r->i];
    d[1] = pos[3 * r->j + 1] - pos[3 * r->i + 1];
    d[2] = pos[3 * r->j + 2] - pos[3 * r->i + 2];
    orc_mic(d, &c);
    r->dx = d[0]; r->dy = d[1]; r->dz = d[2];
    r->gx = 0.0; r->gy = 0.0; r->gz = 0.0;
  }
}

/* Layer 1 back: relative-vector gradients into gpos and the virial.
 * yaff/pes/dlist.c:44-69. */
void orc_dlist_back(double *gpos, double *vtens, const orc_delta *dl, int64_t n) {
  int64_t k;
  for (k = 0; k < n; k++) {
    const orc_delta *r = dl + k;
    if (gpos) {
      gpos[3 * r->j] += r->gx; gpos[3 * r->j + 1] += r->gy; gpos[3 * r->j + 2] += r->gz;
      gpos[3 * r->i] -= r->gx; gpos[3 * r->i + 1] -= r->gy; gpos[3 * r->i + 2] -= r->gz;
    }
    if (vtens) {
      vtens[0] += r->gx * r->dx; vtens[1] += r->gy * r->dx; vtens[2] += r->gz * r->dx;
      vtens[3] += r->gx * r->dy; vtens[4] += r->gy * r->dy; vtens[5] += r->gz * r->dy;
      vtens[6] += r->gx * r->dz; vtens[7] += r->gy * r->dz; vtens[8] += r->gz * r->dz;
    }
  }
}

/* Internal coordinates and valence terms.  Every kind of the reference's
 * tables is restated here: iclist.c:31-320 (forward), :325-858 (back);
 * vlist.c:30-155 (forward), :160-265 (back).  The arithmetic is written in
 * the reference's evaluation order (operand order of every sum and product),
 * so the results agree bit for bit with the reference build. */

static double orc_dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* o = a x b */
static void orc_cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Vector (dx, dy, dz) and gradient (gx, gy, gz) of a delta row. */
#define ORC_D(r) (&(r)->dx)
#define ORC_G(r) (&(r)->gx)

/* ---- forward ---- */

/* Bond length (kinds 0 and 5).  yaff/pes/iclist.c:31-35. */
static double orc_ic_bond(const orc_ic *ic, const orc_delta *dl) {
  const double *d = ORC_D(dl + ic->i0);
  return sqrt(orc_dot3(d, d));
}

/* Cosine of the bend angle (kind 1).  yaff/pes/iclist.c:37-47. */
static double orc_ic_bendcos(const orc_ic *ic, const orc_delta *dl) {
  const double *a = ORC_D(dl + ic->i0), *b = ORC_D(dl + ic->i1);
  double da = sqrt(orc_dot3(a, a));
  double db = sqrt(orc_dot3(b, b));
  double dot;
  if (da == 0 || db == 0) return 0.0;
  dot = orc_dot3(a, b);
  return ic->sign0 * ic->sign1 * dot / da / db;
}

/* Cosine of the dihedral angle from the components of the outer deltas
 * orthogonal to the central one (kind 3).  yaff/pes/iclist.c:57-76. */
static double orc_ic_dihedcos(const orc_ic *ic, const orc_delta *dl) {
  const double *d0 = ORC_D(dl + ic->i0), *d1 = ORC_D(dl + ic->i1), *d2 = ORC_D(dl + ic->i2);
  double a[3], b[3], n1, p0, p2, na, nb;
  int k;
  n1 = sqrt(orc_dot3(d1, d1));
  p0 = orc_dot3(d0, d1) / n1;
  p2 = orc_dot3(d1, d2) / n1;
  for (k = 0; k < 3; k++) {
    a[k] = d0[k] - p0 * d1[k] / n1;
    b[k] = d2[k] - p2 * d1[k] / n1;
  }
  na = sqrt(orc_dot3(a, a));
  nb = sqrt(orc_dot3(b, b));
  return ic->sign0 * ic->sign2 * orc_dot3(a, b) / na / nb;
}

/* Sine of the dihedral angle, (d1 x d0).d2 |d1| / |d1 x d0| / |d2 x d1|;
 * used by the dihedral angle near 0 and pi.  yaff/pes/iclist.c:78-109. */
static double orc_ic_dihedsin(const orc_ic *ic, const orc_delta *dl) {
  const double *d0 = ORC_D(dl + ic->i0), *d1 = ORC_D(dl + ic->i1), *d2 = ORC_D(dl + ic->i2);
  double a[3], b[3], r1, ra, rb;
  orc_cross3(d1, d0, a);
  orc_cross3(d2, d1, b);
  r1 = sqrt(orc_dot3(d1, d1));
  ra = sqrt(orc_dot3(a, a));
  rb = sqrt(orc_dot3(b, b));
  return ic->sign0 * ic->sign1 * ic->sign2 * orc_dot3(a, d2) * r1 / ra / rb;
}

/* d0 . (d1 x d2) times the three delta signs. */
static double orc_dihed_det(const orc_ic *ic, const orc_delta *dl) {
  const double *d0 = ORC_D(dl + ic->i0), *d1 = ORC_D(dl + ic->i1), *d2 = ORC_D(dl + ic->i2);
  double c[3], det;
  orc_cross3(d1, d2, c);
  det = orc_dot3(d0, c);
  det *= ic->sign0 * ic->sign1 * ic->sign2;
  return det;
}

/* Signed dihedral angle: acos where |cos| < 1/2, asin otherwise (kind 4).
 * yaff/pes/iclist.c:111-141. */
static double orc_ic_dihedangle(const orc_ic *ic, const orc_delta *dl) {
  double c = orc_ic_dihedcos(ic, dl), phi;
  if (fabs(c) < 0.5) {
    phi = acos(c);
    if (orc_dihed_det(ic, dl) > 0) phi *= -1;
  } else {
    phi = asin(orc_ic_dihedsin(ic, dl));
    if (c < 0) {
      phi *= -1;
      if (phi > 0) phi -= 0.5 * ORC_TWO_PI;
      else phi += 0.5 * ORC_TWO_PI;
    }
  }
  return phi;
}

/* Cosine of the angle between u2 and the plane of u0, u1.
 * yaff/pes/iclist.c:143-158. */
static double orc_oop_cos(const double *u0, const double *u1, const double *u2) {
  double n[3], nsq, usq, nu;
  orc_cross3(u0, u1, n);
  nsq = orc_dot3(n, n);
  usq = orc_dot3(u2, u2);
  nu = orc_dot3(n, u2);
  return sqrt(1.0 - nu * nu / usq / nsq);
}

/* yaff/pes/iclist.c:180-190. */
static double orc_oop_angle(const double *u0, const double *u1, const double *u2) {
  double c = orc_oop_cos(u0, u1, u2);
  if (c > 1) c = 1;
  else if (c < -1) c = -1;
  return acos(c);
}

/* Signed distance of the end of d2 from the plane of d0, d1 (kind 10) and its
 * square (kind 11).  yaff/pes/iclist.c:212-251. */
static double orc_ic_oopdist(const orc_ic *ic, const orc_delta *dl, int squared) {
  const double *d0 = ORC_D(dl + ic->i0), *d1 = ORC_D(dl + ic->i1), *d2 = ORC_D(dl + ic->i2);
  double n[3], nn, nd;
  orc_cross3(d0, d1, n);
  nn = sqrt(orc_dot3(n, n));
  if (nn == 0) return 0.0;
  nd = orc_dot3(n, d2);
  if (squared) {
    nd /= nn;
    return nd * nd;
  }
  return nd / nn * ic->sign0 * ic->sign1 * ic->sign2;
}

/* |d0 x d1|^2 / |d2|^2: squared distance of a point from a line (kind 17).
 * yaff/pes/iclist.c:279-298. */
static double orc_ic_plsq(const orc_ic *ic, const orc_delta *dl) {
  const double *d0 = ORC_D(dl + ic->i0), *d1 = ORC_D(dl + ic->i1), *d2 = ORC_D(dl + ic->i2);
  double n[3];
  orc_cross3(d0, d1, n);
  return orc_dot3(n, n) / orc_dot3(d2, d2);
}

/* Value of one internal coordinate; returns NAN-free results for every kind
 * 0..17, sets *bad for an unknown kind.  yaff/pes/iclist.c:307-312. */
static double orc_ic_value(const orc_ic *ic, const orc_delta *dl, int *bad) {
  const double *d0, *d1, *d2;
  double c, t;
  switch (ic->kind) {
    case 0: case 5: return orc_ic_bond(ic, dl);
    case 1: return orc_ic_bendcos(ic, dl);
    case 2:
      c = orc_ic_bendcos(ic, dl);
      if (c > 1.0) c = 1.0;
      if (c < -1.0) c = -1.0;
      return acos(c);
    case 3: return orc_ic_dihedcos(ic, dl);
    case 4: return orc_ic_dihedangle(ic, dl);
    case 6: case 7: case 8: case 9:
      d0 = ORC_D(dl + ic->i0); d1 = ORC_D(dl + ic->i1); d2 = ORC_D(dl + ic->i2);
      if (ic->kind == 6) return orc_oop_cos(d0, d1, d2);
      if (ic->kind == 8) return orc_oop_angle(d0, d1, d2);
      if (ic->kind == 7) {
        t = orc_oop_cos(d0, d1, d2);
        t += orc_oop_cos(d2, d0, d1);
        t += orc_oop_cos(d1, d2, d0);
      } else {
        t = orc_oop_angle(d0, d1, d2);
        t += orc_oop_angle(d2, d0, d1);
        t += orc_oop_angle(d1, d2, d0);
      }
      return t / 3;
    case 10: return orc_ic_oopdist(ic, dl, 0);
    case 11: return orc_ic_oopdist(ic, dl, 1);
    case 12: c = orc_ic_dihedcos(ic, dl); return 2.0 * c * c - 1.0;
    case 13: c = orc_ic_dihedcos(ic, dl); return c * (4.0 * c * c - 3.0);
    case 14: c = orc_ic_dihedcos(ic, dl); c *= c; return 8.0 * c * (c - 1.0) + 1.0;
    case 15: c = orc_ic_dihedcos(ic, dl); c *= 2.0 * c; return c * (4.0 * c * (c - 3.0) + 9.0) - 1.0;
    case 16: c = orc_ic_plsq(ic, dl); if (c < 0) c = 0.0; return sqrt(c);
    case 17: return orc_ic_plsq(ic, dl);
    default: *bad = 1; return 0.0;
  }
}

/* Layer 2 forward.  yaff/pes/iclist.c:314-320.  Returns -1 for an unknown
 * kind. */
int orc_iclist_forward(const orc_delta *dl, orc_ic *ic, int64_t n) {
  int64_t i;
  int bad = 0;
  for (i = 0; i < n; i++) {
    ic[i].value = orc_ic_value(ic + i, dl, &bad);
    ic[i].grad = 0.0;
  }
  return bad ? -1 : 0;
}

/* ---- back ---- */

/* yaff/pes/iclist.c:335-360. */
static void orc_back_bendcos(const orc_ic *ic, orc_delta *dl, double value, double grad) {
  orc_delta *a = dl + ic->i0, *b = dl + ic->i1;
  double ea[3], eb[3], da, db, fac;
  int k;
  da = sqrt(orc_dot3(ORC_D(a), ORC_D(a)));
  db = sqrt(orc_dot3(ORC_D(b), ORC_D(b)));
  for (k = 0; k < 3; k++) { ea[k] = ORC_D(a)[k] / da; eb[k] = ORC_D(b)[k] / db; }
  fac = ic->sign0 * ic->sign1;
  grad *= fac;
  value *= fac;
  fac = grad / da;
  for (k = 0; k < 3; k++) ORC_G(a)[k] += fac * (eb[k] - value * ea[k]);
  fac = grad / db;
  for (k = 0; k < 3; k++) ORC_G(b)[k] += fac * (ea[k] - value * eb[k]);
}

/* Chain rule of the dihedral cosine through the projected vectors a, b and
 * their Jacobians towards d0, d1, d2.  yaff/pes/iclist.c:366-439. */
static void orc_back_dihedcos(const orc_ic *ic, orc_delta *dl, double value, double grad) {
  orc_delta *r0 = dl + ic->i0, *r1 = dl + ic->i1, *r2 = dl + ic->i2;
  const double *d0 = ORC_D(r0), *d1 = ORC_D(r1), *d2 = ORC_D(r2);
  double a[3], b[3], ga[3], gb[3], ja0[9], ja1[9], jb1[9];
  double n1, nn, n4, p0, p2, na, nb;
  int r, c;
  n1 = sqrt(orc_dot3(d1, d1));
  p0 = orc_dot3(d0, d1);
  p2 = orc_dot3(d1, d2);
  nn = n1 * n1;
  n4 = n1 * n1 * n1 * n1;
  for (r = 0; r < 3; r++) {
    a[r] = d0[r] - p0 * d1[r] / nn;
    b[r] = d2[r] - p2 * d1[r] / nn;
  }
  na = sqrt(orc_dot3(a, a));
  nb = sqrt(orc_dot3(b, b));
  value *= ic->sign0 * ic->sign2;
  grad *= ic->sign0 * ic->sign2;
  for (r = 0; r < 3; r++) {
    ga[r] = (b[r] / nb - value * a[r] / na) / na;
    gb[r] = (a[r] / na - value * b[r] / nb) / nb;
  }
  for (r = 0; r < 3; r++)
    for (c = 0; c < 3; c++) {
      double t = d1[r] * d1[c] / nn;
      double u0 = -(d0[r] * d1[c] / nn), u2 = -(d2[r] * d1[c] / nn);
      ja0[3 * r + c] = (r == c) ? 1 - t : -t;
      if (r == c) {
        u0 = -(p0 / nn) - d0[r] * d1[c] / nn;
        u2 = -(p2 / nn) - d2[r] * d1[c] / nn;
      }
      ja1[3 * r + c] = u0 + 2 * p0 / n4 * d1[r] * d1[c];
      jb1[3 * r + c] = u2 + 2 * p2 / n4 * d1[r] * d1[c];
    }
  for (c = 0; c < 3; c++) {
    ORC_G(r0)[c] += grad * (ga[0] * ja0[c] + ga[1] * ja0[3 + c] + ga[2] * ja0[6 + c]);
    ORC_G(r1)[c] += grad * (ga[0] * ja1[c] + ga[1] * ja1[3 + c] + ga[2] * ja1[6 + c]
                            + gb[0] * jb1[c] + gb[1] * jb1[3 + c] + gb[2] * jb1[6 + c]);
    ORC_G(r2)[c] += grad * (gb[0] * ja0[c] + gb[1] * ja0[3 + c] + gb[2] * ja0[6 + c]);
  }
}

/* Chain rule of the dihedral sine, a product of four factors.
 * yaff/pes/iclist.c:441-510. */
static void orc_back_dihedsin(const orc_ic *ic, orc_delta *dl, double value, double grad) {
  orc_delta *r0 = dl + ic->i0, *r1 = dl + ic->i1, *r2 = dl + ic->i2;
  const double *d0 = ORC_D(r0), *d1 = ORC_D(r1), *d2 = ORC_D(r2);
  double a[3], b[3], c[3], t[3], n1, ra, rb, fac;
  int k;
  orc_cross3(d1, d0, a);
  orc_cross3(d2, d1, b);
  orc_cross3(d0, d2, c);
  n1 = sqrt(orc_dot3(d1, d1));
  ra = sqrt(orc_dot3(a, a));
  rb = sqrt(orc_dot3(b, b));
  value *= ic->sign0 * ic->sign1 * ic->sign2;
  grad *= ic->sign0 * ic->sign1 * ic->sign2;
  /* triple product (d1 x d0).d2 */
  fac = grad * n1 / ra / rb;
  for (k = 0; k < 3; k++) ORC_G(r0)[k] += fac * b[k];
  for (k = 0; k < 3; k++) ORC_G(r1)[k] += fac * c[k];
  for (k = 0; k < 3; k++) ORC_G(r2)[k] += fac * a[k];
  /* |d1| */
  fac = grad * value / n1 / n1;
  for (k = 0; k < 3; k++) ORC_G(r1)[k] += fac * d1[k];
  /* 1/|d1 x d0| */
  fac = grad * value / ra / ra;
  orc_cross3(a, d1, t);
  for (k = 0; k < 3; k++) ORC_G(r0)[k] -= fac * t[k];
  orc_cross3(a, d0, t);
  for (k = 0; k < 3; k++) ORC_G(r1)[k] += fac * t[k];
  /* 1/|d2 x d1| */
  fac = grad * value / rb / rb;
  orc_cross3(b, d2, t);
  for (k = 0; k < 3; k++) ORC_G(r1)[k] -= fac * t[k];
  orc_cross3(b, d1, t);
  for (k = 0; k < 3; k++) ORC_G(r2)[k] += fac * t[k];
}

/* yaff/pes/iclist.c:512-541. */
static void orc_back_dihedangle(const orc_ic *ic, orc_delta *dl, double grad) {
  double c = orc_ic_dihedcos(ic, dl), s, tmp = grad;
  if (fabs(c) < 0.5) {
    s = sqrt(1 - c * c);
    tmp /= -s;
    if (orc_dihed_det(ic, dl) > 0) tmp *= -1;
    orc_back_dihedcos(ic, dl, c, tmp);
  } else {
    s = orc_ic_dihedsin(ic, dl);
    tmp /= c;
    orc_back_dihedsin(ic, dl, s, tmp);
  }
}

/* Gradient of the out-of-plane cosine towards the three deltas.
 * yaff/pes/iclist.c:543-622. */
static void orc_back_oopcos(orc_delta *r0, orc_delta *r1, orc_delta *r2, double value, double grad) {
  const double *d0 = ORC_D(r0), *d1 = ORC_D(r1), *d2 = ORC_D(r2);
  double c01[3], c12[3], c20[3], t[3], nsq, usq, nu, t0, t1, t2;
  int k;
  orc_cross3(d0, d1, c01);
  orc_cross3(d1, d2, c12);
  orc_cross3(d2, d0, c20);
  nsq = orc_dot3(c01, c01);
  usq = orc_dot3(d2, d2);
  nu = orc_dot3(c01, d2);
  t0 = nu / usq / nsq / value;
  t1 = nu / nsq;
  t2 = nu / usq;
  orc_cross3(d1, c01, t);
  for (k = 0; k < 3; k++) ORC_G(r0)[k] += -t0 * grad * (c12[k] - t1 * t[k]);
  orc_cross3(c01, d0, t);
  for (k = 0; k < 3; k++) ORC_G(r1)[k] += -t0 * grad * (c20[k] - t1 * t[k]);
  for (k = 0; k < 3; k++) ORC_G(r2)[k] += -t0 * grad * (c01[k] - t2 * d2[k]);
}

/* yaff/pes/iclist.c:646-650. */
static void orc_back_oopangle(orc_delta *r0, orc_delta *r1, orc_delta *r2, double value, double grad) {
  double s = sin(value);
  if (s != 0.0) s = -grad / s;
  orc_back_oopcos(r0, r1, r2, cos(value), s);
}

/* Signed out-of-plane distance (squared = 0) and its square (squared = 1).
 * yaff/pes/iclist.c:674-754. */
static void orc_back_oopdist(const orc_ic *ic, orc_delta *dl, double grad, int squared) {
  orc_delta *r0 = dl + ic->i0, *r1 = dl + ic->i1, *r2 = dl + ic->i2;
  const double *d0 = ORC_D(r0), *d1 = ORC_D(r1), *d2 = ORC_D(r2);
  double c01[3], c12[3], c20[3], t[3], nn, nd, fac, t0;
  int k;
  orc_cross3(d0, d1, c01);
  orc_cross3(d1, d2, c12);
  orc_cross3(d2, d0, c20);
  nn = sqrt(orc_dot3(c01, c01));
  nd = orc_dot3(c01, d2);
  if (squared) fac = 2 * nd / nn * grad / nn;
  else fac = grad / nn * ic->sign0 * ic->sign1 * ic->sign2;
  t0 = nd / nn / nn;
  orc_cross3(d1, c01, t);
  for (k = 0; k < 3; k++) ORC_G(r0)[k] += fac * (c12[k] - t0 * t[k]);
  orc_cross3(c01, d0, t);
  for (k = 0; k < 3; k++) ORC_G(r1)[k] += fac * (c20[k] - t0 * t[k]);
  for (k = 0; k < 3; k++) ORC_G(r2)[k] += fac * c01[k];
}

/* yaff/pes/iclist.c:800-833. */
static void orc_back_plsq(const orc_ic *ic, orc_delta *dl, double grad) {
  orc_delta *r0 = dl + ic->i0, *r1 = dl + ic->i1, *r2 = dl + ic->i2;
  const double *d0 = ORC_D(r0), *d1 = ORC_D(r1), *d2 = ORC_D(r2);
  double n[3], t[3], nsq, usq, fac;
  int k;
  orc_cross3(d0, d1, n);
  nsq = orc_dot3(n, n);
  usq = orc_dot3(d2, d2);
  fac = 2.0 * grad / usq;
  orc_cross3(d1, n, t);
  for (k = 0; k < 3; k++) ORC_G(r0)[k] += fac * t[k];
  orc_cross3(d0, n, t);
  for (k = 0; k < 3; k++) ORC_G(r1)[k] -= fac * t[k];
  fac = 2.0 * grad * nsq / (usq * usq);
  for (k = 0; k < 3; k++) ORC_G(r2)[k] -= fac * d2[k];
}

/* Layer 2 back (chain rule into relative-vector gradients), every kind.
 * yaff/pes/iclist.c:325-858. */
int orc_iclist_back(orc_delta *dl, const orc_ic *ic, int64_t n) {
  int64_t i;
  for (i = 0; i < n; i++) {
    const orc_ic *c = ic + i;
    double g = c->grad, v = c->value, x;
    int k;
    switch (c->kind) {
      case 0: case 5: {
        orc_delta *d = dl + c->i0;
        x = g / v;
        for (k = 0; k < 3; k++) ORC_G(d)[k] += x * ORC_D(d)[k];
        break;
      }
      case 1: orc_back_bendcos(c, dl, v, g); break;
      case 2: orc_back_bendcos(c, dl, cos(v), -g / sin(v)); break;
      case 3: orc_back_dihedcos(c, dl, v, g); break;
      case 4: orc_back_dihedangle(c, dl, g); break;
      case 6: orc_back_oopcos(dl + c->i0, dl + c->i1, dl + c->i2, v, g); break;
      case 8: orc_back_oopangle(dl + c->i0, dl + c->i1, dl + c->i2, v, g); break;
      case 7: case 9: {
        orc_delta *r0 = dl + c->i0, *r1 = dl + c->i1, *r2 = dl + c->i2;
        orc_delta *rot[3][3] = {{r0, r1, r2}, {r2, r0, r1}, {r1, r2, r0}};
        for (k = 0; k < 3; k++) {
          const double *u0 = ORC_D(rot[k][0]), *u1 = ORC_D(rot[k][1]), *u2 = ORC_D(rot[k][2]);
          if (c->kind == 7)
            orc_back_oopcos(rot[k][0], rot[k][1], rot[k][2], orc_oop_cos(u0, u1, u2), g / 3.0);
          else
            orc_back_oopangle(rot[k][0], rot[k][1], rot[k][2], orc_oop_angle(u0, u1, u2), g / 3.0);
        }
        break;
      }
      case 10: orc_back_oopdist(c, dl, g, 0); break;
      case 11: orc_back_oopdist(c, dl, g, 1); break;
      case 12: case 13: case 14: case 15: {
        double cc = orc_ic_dihedcos(c, dl), t;
        if (c->kind == 12) t = 4.0 * cc * g;
        else if (c->kind == 13) t = (12.0 * cc * cc - 3.0) * g;
        else if (c->kind == 14) t = 16.0 * cc * (2.0 * cc * cc - 1.0) * g;
        else t = 12.0 * cc * (16.0 * cc * cc * (cc * cc - 1.0) + 3.0) * g;
        orc_back_dihedcos(c, dl, cc, t);
        break;
      }
      case 16:
        x = (v == 0.0) ? 0.0 : 0.5 * g / v;
        orc_back_plsq(c, dl, x);
        break;
      case 17: orc_back_plsq(c, dl, g); break;
      default: return -1;
    }
  }
  return 0;
}

/* ---- layer 3: energy terms ---- */

/* Energy of one term.  yaff/pes/vlist.c:30-144 (kinds 0..15). */
static double orc_vterm_energy(const orc_vterm *t, const orc_ic *ic) {
  double q = ic[t->ic0].value, x, x2, c, K, y;
  switch (t->kind) {
    case 0: x = q - t->par1; return 0.5 * (t->par0) * x * x;
    case 1: return t->par0 * q + t->par1 * q * q + t->par2 * q * q * q + t->par3 * q * q * q * q;
    case 2: x = t->par1 / q; return 0.5 * t->par0 * t->par1 * t->par1 * (1.0 + x * (x - 2.0));
    case 3: return t->par0 * (q - t->par1) * (ic[t->ic1].value - t->par2);
    case 4: return 0.5 * t->par1 * (1 - cos(t->par0 * (q - t->par2)));
    case 5: return 0.5 * t->par0 * (1 + t->par1 * q);
    case 6: c = q; return 0.5 * t->par0 * (1 + t->par1 * (2 * c * c - 1));
    case 7: c = q; return 0.5 * t->par0 * (1 + t->par1 * c * (4 * c * c - 3));
    case 8: c = q * q; return 0.5 * t->par0 * (1 + t->par1 * (8 * c * c - 8 * c + 1));
    case 9: c = q * q; return 0.5 * t->par0 * (1 + t->par1 * (32 * c * c * c - 48 * c * c + 18 * c - 1));
    case 10:
      return t->par0 * q + t->par1 * q * q + t->par2 * q * q * q + t->par3 * q * q * q * q +
             t->par4 * q * q * q * q * q + t->par5 * q * q * q * q * q * q;
    case 11:
      x = q - t->par1; x2 = x * x;
      return 0.5 * (t->par0) * x2 * (1.0 - 1.349402 * x + 1.062183 * x2);
    case 12:
      x = q - t->par1; x2 = x * x;
      return 0.5 * (t->par0) * x2 * (1.0 - 0.802141 * x + 0.183837 * x2 - 0.131664 * x2 * x + 0.237090 * x2 * x2);
    case 13:
      K = (t->par1 - t->par2) * (t->par1 - t->par2);
      K *= K;
      K = t->par0 / K;
      x = q - t->par1;
      y = q - t->par2;
      y *= y;
      return 0.5 * K * x * x * y * y;
    case 14: x = t->par1 * (q - t->par2); return t->par0 * (exp(-2.0 * x) - 2.0 * exp(-x));
    case 15:
      x = q - t->par5;
      return t->par0 + t->par1 * x + t->par2 * x * x + t->par3 * x * x * x + t->par4 * x * x * x * x;
    default: return NAN;
  }
}

/* Layer 3 forward, sequential sum.  yaff/pes/vlist.c:146-155. */
double orc_vlist_forward(const orc_ic *ic, orc_vterm *vt, int64_t n) {
  int64_t i;
  double e = 0.0;
  for (i = 0; i < n; i++) {
    vt[i].energy = orc_vterm_energy(vt + i, ic);
    e += vt[i].energy;
  }
  return e;
}

/* Layer 3 back: dE/dq added to the coordinates' grad.
 * yaff/pes/vlist.c:160-265. */
void orc_vlist_back(orc_ic *ic, const orc_vterm *vt, int64_t n) {
  int64_t i;
  for (i = 0; i < n; i++) {
    const orc_vterm *t = vt + i;
    double q = ic[t->ic0].value, x, q2, c, K, y, z;
    double *g = &ic[t->ic0].grad;
    switch (t->kind) {
      case 0: *g += (t->par0) * (q - t->par1); break;
      case 1: *g += t->par0 + 2.0 * t->par1 * q + 3.0 * t->par2 * q * q + 4.0 * t->par3 * q * q * q; break;
      case 2: x = t->par1 / q; *g += t->par0 * t->par1 * (x * x - x * x * x); break;
      case 3:
        *g += t->par0 * (ic[t->ic1].value - t->par2);
        ic[t->ic1].grad += t->par0 * (ic[t->ic0].value - t->par1);
        break;
      case 4: *g += 0.5 * t->par1 * t->par0 * sin(t->par0 * (q - t->par2)); break;
      case 5: *g += 0.5 * t->par0 * t->par1; break;
      case 6: *g += t->par1 * 2.0 * t->par0 * q; break;
      case 7: c = q; *g += t->par1 * 1.5 * t->par0 * (4 * c * c - 1); break;
      case 8: c = q; *g += t->par1 * 8 * t->par0 * c * (2 * c * c - 1); break;
      case 9: c = q; *g += t->par1 * 6 * t->par0 * c * (16 * c * c * c * c - 16 * c * c + 3); break;
      case 10:
        *g += t->par0 + 2.0 * t->par1 * q + 3.0 * t->par2 * q * q + 4.0 * t->par3 * q * q * q +
              5.0 * t->par4 * q * q * q * q + 6.0 * t->par5 * q * q * q * q * q;
        break;
      case 11: x = q - t->par1; *g += (t->par0) * (x - 2.024103 * x * x + 2.124366 * x * x * x); break;
      case 12:
        x = q - t->par1; q2 = x * x;
        *g += (t->par0) * (x - 1.203211 * q2 + 0.367674 * q2 * x - 0.329159 * q2 * q2 + 0.711270 * q2 * q2 * x);
        break;
      case 13:
        K = (t->par1 - t->par2) * (t->par1 - t->par2);
        K *= K;
        K = t->par0 / (K);
        x = q - t->par1;
        y = q - t->par2;
        y *= y;
        z = q - t->par2;
        *g += 0.5 * K * (2 * x * y * y + 4 * x * x * y * z);
        break;
      case 14: x = t->par1 * (q - t->par2); *g += -2.0 * t->par1 * t->par0 * (exp(-2.0 * x) - exp(-x)); break;
      case 15: x = q - t->par5; *g += t->par1 + 2.0 * t->par2 * x + 3.0 * t->par3 * x * x + 4.0 * t->par4 * x * x * x; break;
      default: break;
    }
  }
}
