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
int64_t orc_nlist_build(const double *pos, int64_t natom, double rcut,
                        const int64_t *rmax, const double *rv, const double *gv,
                        int nvec, int64_t nlow, int64_t nhigh,
                        orc_neigh *out, int64_t cap) {
  orc_cell c;
  int64_t a, b, n = 0, k;
  double rc2 = rcut * rcut;
  for (k = 0; k < 9; k++) { c.rv[k] = rv[k]; c.gv[k] = gv[k]; }
  c.nvec = nvec;
  for (a = nlow; a < natom; a++) {
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

enum { ORC_LJ = 0, ORC_MM3 = 1, ORC_EI = 2 };
enum { ORC_TR_NONE = 0, ORC_TR_HAMMER = 1, ORC_TR_SWITCH3 = 2 };

typedef struct {
  int kind;
  const double *sigma, *epsilon;   /* LJ, MM3 */
  const int32_t *onlypauli;        /* MM3 */
  const double *charges, *radii;   /* EI */
  double alpha, dielectric;        /* EI */
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

/* Generic pair loop with exclusion scaling, truncation chain rule, gradient
 * and virial accumulation.  yaff/pes/pair_pot.c:84-176 (pair_pot_compute). */
double orc_pair_compute(const orc_neigh *rows, int64_t n, const orc_scale *st,
                        int64_t nst, int kind, const double *sigma,
                        const double *epsilon, const int32_t *onlypauli,
                        const double *charges, const double *radii,
                        double alpha, double dielectric, double rcut,
                        int tr_kind, double tr_par, double *gpos, double *vtens) {
  orc_pairpot p;
  int64_t i, srow = 0;
  double energy = 0.0;
  p.kind = kind; p.sigma = sigma; p.epsilon = epsilon; p.onlypauli = onlypauli;
  p.charges = charges; p.radii = radii; p.alpha = alpha; p.dielectric = dielectric;
  p.rcut = rcut; p.tr_kind = tr_kind; p.tr_par = tr_par;
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
    if (kind == ORC_LJ) v = orc_lj(&p, r->a, r->b, r->d, want_g ? &vg : NULL);
    else if (kind == ORC_MM3) v = orc_mm3(&p, r->a, r->b, r->d, want_g ? &vg : NULL);
    else v = orc_ei(&p, r->a, r->b, r->d, want_g ? &vg : NULL);
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
double orc_ewald_reci(const double *pos, int64_t natom, int64_t nlow, int64_t nhigh,
                      const double *charges, const double *rv, const double *gv,
                      double volume, double alpha, const int64_t *gmax,
                      double gcut, double dielectric, double *gpos,
                      double *work, double *vtens) {
  double kv[9], energy = 0.0, fac1, fac2, gc2, dfac;
  int64_t g0, g1, g2, i;
  (void)rv;
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
  if (vtens) { vtens[0] -= energy; vtens[4] -= energy; vtens[8] -= energy; }
  dfac = 1.0 / dielectric;
  if (gpos) for (i = 0; i < 3 * natom; i++) gpos[i] *= dfac;
  if (vtens) for (i = 0; i < 9; i++) vtens[i] *= dfac;
  return energy * dfac;
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

/* Bond length (kinds 0 and 5).  yaff/pes/iclist.c:31-35. */
static double orc_ic_bond(const orc_ic *ic, const orc_delta *dl) {
  const orc_delta *d = dl + ic->i0;
  return sqrt(d->dx * d->dx + d->dy * d->dy + d->dz * d->dz);
}

/* Cosine of the bend angle (kind 1).  yaff/pes/iclist.c:37-47. */
static double orc_ic_bendcos(const orc_ic *ic, const orc_delta *dl) {
  const orc_delta *a = dl + ic->i0, *b = dl + ic->i1;
  double da = sqrt(a->dx * a->dx + a->dy * a->dy + a->dz * a->dz);
  double db = sqrt(b->dx * b->dx + b->dy * b->dy + b->dz * b->dz);
  double dot;
  if (da == 0 || db == 0) return 0.0;
  dot = a->dx * b->dx + a->dy * b->dy + a->dz * b->dz;
  return ic->sign0 * ic->sign1 * dot / da / db;
}

/* Layer 2 forward for bond (0), bend cos (1), bend angle (2) and
 * Urey-Bradley (5).  yaff/pes/iclist.c:31-55, :307-320.  Returns -1 if a
 * kind outside that set is present. */
int orc_iclist_forward(const orc_delta *dl, orc_ic *ic, int64_t n) {
  int64_t i;
  for (i = 0; i < n; i++) {
    double v;
    switch (ic[i].kind) {
      case 0: case 5: v = orc_ic_bond(ic + i, dl); break;
      case 1: v = orc_ic_bendcos(ic + i, dl); break;
      case 2:
        v = orc_ic_bendcos(ic + i, dl);
        if (v > 1.0) v = 1.0;
        if (v < -1.0) v = -1.0;
        v = acos(v);
        break;
      default: return -1;
    }
    ic[i].value = v;
    ic[i].grad = 0.0;
  }
  return 0;
}

static void orc_back_bendcos(const orc_ic *ic, orc_delta *dl, double value, double grad) {
  orc_delta *a = dl + ic->i0, *b = dl + ic->i1;
  double ea[3], eb[3], da, db, fac;
  da = sqrt(a->dx * a->dx + a->dy * a->dy + a->dz * a->dz);
  db = sqrt(b->dx * b->dx + b->dy * b->dy + b->dz * b->dz);
  ea[0] = a->dx / da; ea[1] = a->dy / da; ea[2] = a->dz / da;
  eb[0] = b->dx / db; eb[1] = b->dy / db; eb[2] = b->dz / db;
  fac = ic->sign0 * ic->sign1;
  grad *= fac;
  value *= fac;
  fac = grad / da;
  a->gx += fac * (eb[0] - value * ea[0]);
  a->gy += fac * (eb[1] - value * ea[1]);
  a->gz += fac * (eb[2] - value * ea[2]);
  fac = grad / db;
  b->gx += fac * (ea[0] - value * eb[0]);
  b->gy += fac * (ea[1] - value * eb[1]);
  b->gz += fac * (ea[2] - value * eb[2]);
}

/* Layer 2 back (chain rule into relative-vector gradients).
 * yaff/pes/iclist.c:325-364, :853-858. */
int orc_iclist_back(orc_delta *dl, const orc_ic *ic, int64_t n) {
  int64_t i;
  for (i = 0; i < n; i++) {
    const orc_ic *c = ic + i;
    switch (c->kind) {
      case 0: case 5: {
        orc_delta *d = dl + c->i0;
        double x = c->grad / c->value;
        d->gx += x * d->dx; d->gy += x * d->dy; d->gz += x * d->dz;
        break;
      }
      case 1: orc_back_bendcos(c, dl, c->value, c->grad); break;
      case 2: orc_back_bendcos(c, dl, cos(c->value), -c->grad / sin(c->value)); break;
      default: return -1;
    }
  }
  return 0;
}

/* Layer 3: harmonic terms 0.5 K (q - q0)^2 (kind 0).
 * yaff/pes/vlist.c:30-34, :146-155, :160-162, :260-265. */
double orc_vlist_forward(const orc_ic *ic, orc_vterm *vt, int64_t n) {
  int64_t i;
  double e = 0.0;
  for (i = 0; i < n; i++) {
    double x = ic[vt[i].ic0].value - vt[i].par1;
    vt[i].energy = 0.5 * (vt[i].par0) * x * x;
    e += vt[i].energy;
  }
  return e;
}

void orc_vlist_back(orc_ic *ic, const orc_vterm *vt, int64_t n) {
  int64_t i;
  for (i = 0; i < n; i++)
    ic[vt[i].ic0].grad += (vt[i].par0) * (ic[vt[i].ic0].value - vt[i].par1);
}
