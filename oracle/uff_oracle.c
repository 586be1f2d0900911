/*
 * uff_oracle.c -- FP64 CPU oracle for the MMO UFF scoring hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the CPU baseline
 * timed by bench.py.  The shipped library never links or calls this file.
 * Each function cites the reference OCaml it restates (paths inside
 * UnixJunkie/MMO).  Parity against the reference itself is unpinned (no golden
 * energies ship with it); see uff_oracle.h for what pins this oracle.
 */
#include "uff_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* const.ml:12-18 and UFF.ml:25 */
static const double CUTOFF = 12.0;
static const double EPS_PROT = 4.0;
double orc_elec_weight(void) { return 332.0637 / EPS_PROT; }

/* UFF.ml:10-22: (anum, x_i, D_i); anum 0 is a virtual element with no vdW */
static const struct { int anum; double xi, di; } UFF_TABLE[] = {
    {0, 0.0, 0.0},     {1, 2.886, 0.044},  {6, 3.851, 0.105},  {7, 3.660, 0.069},
    {8, 3.500, 0.060}, {9, 3.364, 0.050},  {12, 3.021, 0.111}, {15, 4.147, 0.305},
    {16, 4.035, 0.274}, {17, 3.947, 0.227}, {35, 4.189, 0.251}, {53, 4.500, 0.339}};

int orc_uff_params(int anum, double *xi, double *di) {
  for (unsigned k = 0; k < sizeof(UFF_TABLE) / sizeof(UFF_TABLE[0]); ++k)
    if (UFF_TABLE[k].anum == anum) {
      *xi = UFF_TABLE[k].xi;
      *di = UFF_TABLE[k].di;
      return 1;
    }
  return 0;
}

/* UFF.ml:43-51 (FF.geo_mean for both); the table holds NaN for unsupported
 * elements (UFF.ml:37), which the NaN returned here reproduces. */
void orc_pair_params(const orc_physics *ph, int a1, int a2, double *x_ij, double *d_ij) {
  double x1, d1, x2, d2;
  if (!orc_uff_params(a1, &x1, &d1) || !orc_uff_params(a2, &x2, &d2)) {
    *x_ij = NAN;
    *d_ij = NAN;
    return;
  }
  *x_ij = ph->mixing == 1 ? 0.5 * (x1 + x2) : sqrt(x1 * x2);
  *d_ij = sqrt(d1 * d2);
}

/* FF.ml:17-20 */
double orc_shift_12A(double d) {
  if (d < 12.0) {
    double s = 1.0 - (d / 12.0) * (d / 12.0);
    return s * s;
  }
  return 0.0;
}

/* math.ml:58-62 */
double orc_non_zero_dist(double d) { return d < 0.01 ? 0.01 : d; }

/* FF.ml:5-12: pow6 x = pow3 (x * x) */
static double pow6(double x) {
  double x2 = x * x;
  return x2 * x2 * x2;
}

static void cross(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* math.ml:48-56: atan2((u1 |u2|) . (u2 x u3), (u1 x u2) . (u2 x u3)) */
double orc_dihedral(const double i[3], const double j[3], const double k[3], const double l[3]) {
  double u1[3], u2[3], u3[3], u2u3[3], u1u2[3], u1m[3];
  for (int d = 0; d < 3; ++d) {
    u1[d] = j[d] - i[d];
    u2[d] = k[d] - j[d];
    u3[d] = l[d] - k[d];
  }
  cross(u2, u3, u2u3);
  double m2 = sqrt(dot(u2, u2));
  for (int d = 0; d < 3; ++d) u1m[d] = u1[d] * m2;
  cross(u1, u2, u1u2);
  return atan2(dot(u1m, u2u3), dot(u1u2, u2u3));
}

/* rot.ml:52-66: R = Rz(g) Ry(b) Rx(a), row-major a..i */
void orc_rot_xyz(double al, double be, double ga, double R[9]) {
  double ca = cos(al), sa = sin(al), cb = cos(be), sb = sin(be), cg = cos(ga), sg = sin(ga);
  R[0] = cb * cg;
  R[1] = cg * sa * sb - ca * sg;
  R[2] = sa * sg + ca * cg * sb;
  R[3] = cb * sg;
  R[4] = ca * cg + sa * sb * sg;
  R[5] = ca * sb * sg - cg * sa;
  R[6] = -sb;
  R[7] = cb * sa;
  R[8] = ca * cb;
}

/* d R / d(a, b, g), entry by entry from the closed form above */
static void rot_xyz_derivs(double al, double be, double ga, double dA[9], double dB[9],
                           double dG[9]) {
  double ca = cos(al), sa = sin(al), cb = cos(be), sb = sin(be), cg = cos(ga), sg = sin(ga);
  dA[0] = 0.0;
  dA[1] = cg * ca * sb + sa * sg;
  dA[2] = ca * sg - sa * cg * sb;
  dA[3] = 0.0;
  dA[4] = -sa * cg + ca * sb * sg;
  dA[5] = -sa * sb * sg - cg * ca;
  dA[6] = 0.0;
  dA[7] = cb * ca;
  dA[8] = -sa * cb;

  dB[0] = -sb * cg;
  dB[1] = cg * sa * cb;
  dB[2] = ca * cg * cb;
  dB[3] = -sb * sg;
  dB[4] = sa * cb * sg;
  dB[5] = ca * cb * sg;
  dB[6] = -cb;
  dB[7] = -sb * sa;
  dB[8] = -ca * sb;

  dG[0] = -cb * sg;
  dG[1] = -sg * sa * sb - ca * cg;
  dG[2] = sa * cg - ca * sg * sb;
  dG[3] = cb * cg;
  dG[4] = -ca * sg + sa * sb * cg;
  dG[5] = ca * sb * cg + sg * sa;
  dG[6] = 0.0;
  dG[7] = 0.0;
  dG[8] = 0.0;
}

/* rot.ml:136-146 */
void orc_rot_axis_angle(const double u[3], double theta, double R[9]) {
  double c = cos(theta), s = sin(theta), o = 1.0 - c;
  double x = u[0], y = u[1], z = u[2];
  R[0] = c + x * x * o;
  R[1] = x * y * o - z * s;
  R[2] = x * z * o + y * s;
  R[3] = x * y * o + z * s;
  R[4] = c + y * y * o;
  R[5] = y * z * o - x * s;
  R[6] = x * z * o - y * s;
  R[7] = y * z * o + x * s;
  R[8] = c + z * z * o;
}

static void matvec(const double R[9], const double v[3], double o[3]) {
  o[0] = R[0] * v[0] + R[1] * v[1] + R[2] * v[2];
  o[1] = R[3] * v[0] + R[4] * v[1] + R[5] * v[2];
  o[2] = R[6] * v[0] + R[7] * v[1] + R[8] * v[2];
}
static void matTvec(const double R[9], const double v[3], double o[3]) {
  o[0] = R[0] * v[0] + R[3] * v[1] + R[6] * v[2];
  o[1] = R[1] * v[0] + R[4] * v[1] + R[7] * v[2];
  o[2] = R[2] * v[0] + R[5] * v[1] + R[8] * v[2];
}

/* bond axis of mol.ml:615-619: normalize (p_right - p_left) */
static void bond_axis(const double *x, const double *y, const double *z, int left, int right,
                      double c[3], double a[3], double u[3], double *alen) {
  c[0] = x[right];
  c[1] = y[right];
  c[2] = z[right];
  a[0] = c[0] - x[left];
  a[1] = c[1] - y[left];
  a[2] = c[2] - z[left];
  *alen = sqrt(dot(a, a));
  u[0] = a[0] / *alen;
  u[1] = a[1] / *alen;
  u[2] = a[2] / *alen;
}

/* mol.ml:610-631 */
void orc_rotate_bond(int n, double *x, double *y, double *z, int left, int right,
                     const int *grp, int ng, double alpha) {
  (void)n;
  double c[3], a[3], u[3], alen, R[9];
  bond_axis(x, y, z, left, right, c, a, u, &alen);
  orc_rot_axis_angle(u, alpha, R);
  for (int k = 0; k < ng; ++k) {
    int i = grp[k];
    double v[3] = {x[i] - c[0], y[i] - c[1], z[i] - c[2]}, w[3];
    matvec(R, v, w);
    x[i] = w[0] + c[0];
    y[i] = w[1] + c[1];
    z[i] = w[2] + c[2];
  }
}

static void centroid(int n, const double *x, const double *y, const double *z, double c[3]) {
  double sx = 0, sy = 0, sz = 0;
  for (int i = 0; i < n; ++i) {
    sx += x[i];
    sy += y[i];
    sz += z[i];
  }
  c[0] = sx / n;
  c[1] = sy / n;
  c[2] = sz / n;
}

/* mol.ml:576-591: radius = max_i (0.01 + |center - x_i|); Too_long above 12 A */
static int too_long(int n, const double *x, const double *y, const double *z) {
  if (n == 0) return 0;
  double c[3], r = 0.0;
  centroid(n, x, y, z, c);
  for (int i = 0; i < n; ++i) {
    double dx = c[0] - x[i], dy = c[1] - y[i], dz = c[2] - z[i];
    double d = 0.01 + sqrt(dx * dx + dy * dy + dz * dz);
    if (d > r) r = d;
  }
  return r > CUTOFF;
}

/* torsions of optim.ml:68-71 applied in bond order; returns Too_long status */
static int apply_torsions(const orc_ligand *lig, const double *tau, double *x, double *y,
                          double *z) {
  int n = lig->m.n;
  memcpy(x, lig->m.x, sizeof(double) * n);
  memcpy(y, lig->m.y, sizeof(double) * n);
  memcpy(z, lig->m.z, sizeof(double) * n);
  for (int t = 0; t < lig->nrb; ++t)
    orc_rotate_bond(n, x, y, z, lig->bond_lr[2 * t], lig->bond_lr[2 * t + 1],
                    lig->grp_atoms + lig->grp_off[t], lig->grp_off[t + 1] - lig->grp_off[t],
                    tau[t]);
  return too_long(n, x, y, z) ? ORC_S_TOO_LONG : 0;
}

/* optim.ml:64-80 (flags without RECENTER) or mol.ml:705-710 (RECENTER) */
int orc_apply_config(const orc_ligand *lig, const double *conf, int flags, double *x,
                     double *y, double *z) {
  int n = lig->m.n;
  int st = apply_torsions(lig, conf + 6, x, y, z);
  double R[9], c[3] = {0, 0, 0};
  orc_rot_xyz(conf[3], conf[4], conf[5], R);
  if (flags & ORC_F_RECENTER) centroid(n, x, y, z, c);
  for (int i = 0; i < n; ++i) {
    double v[3] = {x[i] - c[0], y[i] - c[1], z[i] - c[2]}, w[3];
    matvec(R, v, w);
    x[i] = w[0] + conf[0];
    y[i] = w[1] + conf[1];
    z[i] = w[2] + conf[2];
  }
  return st;
}

/* one pair term before the elec weight: elec part and vdW part, FP64, in the
 * operation order of mol.ml:840-845 */
static inline void pair_terms(int dielectric, double r, double q_i, double q_j, double x_ij,
                              double d_ij, double w, double *el, double *vdw) {
  double p6 = pow6(x_ij / r);
  double qq = q_i * q_j;
  *el = w * (dielectric == 1 ? qq / (r * r) : qq / r);
  *vdw = w * (d_ij * ((-2.0 * p6) + (p6 * p6)));
}

/* mol.ml:796-818 (global) and mol.ml:822-849 (shifted); protein-major order */
void orc_ene_inter_parts(const orc_physics *ph, const orc_mol *prot, const orc_mol *lig,
                         double parts[2]) {
  double se = 0.0, sv = 0.0;
  for (int i = 0; i < prot->n; ++i) {
    for (int j = 0; j < lig->n; ++j) {
      double dx = prot->x[i] - lig->x[j], dy = prot->y[i] - lig->y[j],
             dz = prot->z[i] - lig->z[j];
      double r2 = dx * dx + dy * dy + dz * dz;
      double w = 1.0, r;
      if (ph->inter_form == 0) {
        if (!(r2 < 144.0)) continue;
        r = orc_non_zero_dist(sqrt(r2));
        w = orc_shift_12A(r);
      } else {
        r = orc_non_zero_dist(sqrt(r2));
      }
      double x_ij, d_ij, el, vdw;
      orc_pair_params(ph, prot->anum[i], lig->anum[j], &x_ij, &d_ij);
      pair_terms(ph->dielectric, r, prot->q[i], lig->q[j], x_ij, d_ij, w, &el, &vdw);
      se += el;
      sv += vdw;
    }
  }
  parts[0] = orc_elec_weight() * se;
  parts[1] = sv;
}

double orc_ene_inter(const orc_physics *ph, const orc_mol *prot, const orc_mol *lig) {
  double p[2];
  orc_ene_inter_parts(ph, prot, lig, p);
  return p[0] + p[1];
}

/* mol.ml:881-903 (plain) and mol.ml:853-877 (shifted, 12 A) */
double orc_ene_intra(const orc_physics *ph, const orc_mol *lig, const uint8_t *interacting) {
  int n = lig->n;
  double se = 0.0, sv = 0.0;
  for (int i = 0; i < n - 1; ++i) {
    for (int j = i + 1; j < n; ++j) {
      if (!interacting[i * n + j]) continue;
      double dx = lig->x[i] - lig->x[j], dy = lig->y[i] - lig->y[j], dz = lig->z[i] - lig->z[j];
      double r = orc_non_zero_dist(sqrt(dx * dx + dy * dy + dz * dz));
      double w = 1.0;
      if (ph->intra_form == 1) {
        if (!(r < 12.0)) continue;
        w = orc_shift_12A(r);
      }
      double x_ij, d_ij, el, vdw;
      orc_pair_params(ph, lig->anum[i], lig->anum[j], &x_ij, &d_ij);
      pair_terms(ph->dielectric, r, lig->q[i], lig->q[j], x_ij, d_ij, w, &el, &vdw);
      se += el;
      sv += vdw;
    }
  }
  return orc_elec_weight() * se + sv;
}

/* ---- cell grid: the 12 A neighbour query of mol.ml:939 -------------------- */
struct orc_cells {
  orc_mol prot;
  double lo[3];
  int dim[3];
  int *start; /* dim0*dim1*dim2 + 1 */
  int *idx;   /* protein atoms sorted by cell */
};

static int cell_coord(double v, double lo, int dim) {
  int c = (int)floor((v - lo) / CUTOFF);
  if (c < 0) c = 0;
  if (c >= dim) c = dim - 1;
  return c;
}

orc_cells *orc_cells_build(const orc_mol *prot) {
  orc_cells *c = (orc_cells *)calloc(1, sizeof(orc_cells));
  c->prot = *prot;
  double hi[3] = {-1e300, -1e300, -1e300};
  c->lo[0] = c->lo[1] = c->lo[2] = 1e300;
  const double *xyz[3] = {prot->x, prot->y, prot->z};
  for (int i = 0; i < prot->n; ++i)
    for (int d = 0; d < 3; ++d) {
      if (xyz[d][i] < c->lo[d]) c->lo[d] = xyz[d][i];
      if (xyz[d][i] > hi[d]) hi[d] = xyz[d][i];
    }
  if (prot->n == 0) c->lo[0] = c->lo[1] = c->lo[2] = hi[0] = hi[1] = hi[2] = 0.0;
  for (int d = 0; d < 3; ++d) c->dim[d] = (int)floor((hi[d] - c->lo[d]) / CUTOFF) + 1;
  int ncell = c->dim[0] * c->dim[1] * c->dim[2];
  c->start = (int *)calloc((size_t)(ncell > 0 ? ncell : 1) + 1, sizeof(int));
  c->idx = (int *)malloc(sizeof(int) * (prot->n > 0 ? prot->n : 1));
  int *cid = (int *)malloc(sizeof(int) * (prot->n > 0 ? prot->n : 1));
  for (int i = 0; i < prot->n; ++i) {
    int cx = cell_coord(prot->x[i], c->lo[0], c->dim[0]);
    int cy = cell_coord(prot->y[i], c->lo[1], c->dim[1]);
    int cz = cell_coord(prot->z[i], c->lo[2], c->dim[2]);
    cid[i] = (cz * c->dim[1] + cy) * c->dim[0] + cx;
    c->start[cid[i] + 1]++;
  }
  for (int k = 0; k < ncell; ++k) c->start[k + 1] += c->start[k];
  int *fill = (int *)calloc((size_t)(ncell > 0 ? ncell : 1), sizeof(int));
  for (int i = 0; i < prot->n; ++i) c->idx[c->start[cid[i]] + fill[cid[i]]++] = i;
  free(fill);
  free(cid);
  return c;
}

void orc_cells_free(orc_cells *c) {
  if (!c) return;
  free(c->start);
  free(c->idx);
  free(c);
}

/* mol.ml:928-960: ligand-major; protein atoms within 12 A of each ligand atom.
 * The shifted weight is 0 at 12 A, so this equals the brute shifted sum up to
 * summation order. */
double orc_ene_inter_cells(const orc_physics *ph, const orc_cells *c, const orc_mol *lig) {
  const orc_mol *prot = &c->prot;
  double se = 0.0, sv = 0.0;
  for (int j = 0; j < lig->n; ++j) {
    int cx = (int)floor((lig->x[j] - c->lo[0]) / CUTOFF);
    int cy = (int)floor((lig->y[j] - c->lo[1]) / CUTOFF);
    int cz = (int)floor((lig->z[j] - c->lo[2]) / CUTOFF);
    for (int gz = cz - 1; gz <= cz + 1; ++gz) {
      if (gz < 0 || gz >= c->dim[2]) continue;
      for (int gy = cy - 1; gy <= cy + 1; ++gy) {
        if (gy < 0 || gy >= c->dim[1]) continue;
        for (int gx = cx - 1; gx <= cx + 1; ++gx) {
          if (gx < 0 || gx >= c->dim[0]) continue;
          int cell = (gz * c->dim[1] + gy) * c->dim[0] + gx;
          for (int k = c->start[cell]; k < c->start[cell + 1]; ++k) {
            int i = c->idx[k];
            double dx = prot->x[i] - lig->x[j], dy = prot->y[i] - lig->y[j],
                   dz = prot->z[i] - lig->z[j];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 < 144.0)) continue;
            double r = orc_non_zero_dist(sqrt(r2));
            double w = orc_shift_12A(r);
            double x_ij, d_ij, el, vdw;
            orc_pair_params(ph, lig->anum[j], prot->anum[i], &x_ij, &d_ij);
            pair_terms(ph->dielectric, r, prot->q[i], lig->q[j], x_ij, d_ij, w, &el, &vdw);
            se += el;
            sv += vdw;
          }
        }
      }
    }
  }
  return orc_elec_weight() * se + sv;
}

double orc_score_conf(const orc_physics *ph, const orc_mol *prot, const orc_cells *cells,
                      const orc_ligand *lig, const double *conf, int flags, int *status) {
  int n = lig->m.n;
  double *buf = (double *)malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
  double *x = buf, *y = buf + n, *z = buf + 2 * n;
  int st = orc_apply_config(lig, conf, flags, x, y, z);
  orc_mol m = lig->m;
  m.x = x;
  m.y = y;
  m.z = z;
  double E = 0.0;
  if (flags & ORC_F_INTER)
    E += (cells && ph->inter_form == 0) ? orc_ene_inter_cells(ph, cells, &m)
                                        : orc_ene_inter(ph, prot, &m);
  if (flags & ORC_F_INTRA) E += orc_ene_intra(ph, &m, lig->interacting);
  if (!isfinite(E)) st |= ORC_S_NONFINITE;
  if (status) *status = st;
  free(buf);
  return E;
}

/* lds.ml:1118-1136 */
void orc_grad_fd(const orc_physics *ph, const orc_mol *prot, const orc_cells *cells,
                 const orc_ligand *lig, const double *conf, int flags, const double *eps,
                 double *grad) {
  int nd = 6 + lig->nrb;
  double *c = (double *)malloc(sizeof(double) * nd);
  memcpy(c, conf, sizeof(double) * nd);
  for (int k = 0; k < nd; ++k) {
    c[k] = conf[k] - eps[k];
    double before = orc_score_conf(ph, prot, cells, lig, c, flags, NULL);
    c[k] = conf[k] + eps[k];
    double after = orc_score_conf(ph, prot, cells, lig, c, flags, NULL);
    c[k] = conf[k];
    grad[k] = (after - before) / (2.0 * eps[k]);
  }
  free(c);
}

/* d(pair energy)/d(r2) * 2 for one pair with the switch weight; the pair
 * energy is w(r) * (D p6 (p6 - 2) + K qq / r^m), r = max(|d|, 0.01).  Below
 * 0.01 A the distance is clamped, so the derivative there is zero. */
static double pair_energy_grad(int dielectric, int shifted, double r2, double qqK, double x_ij,
                               double d_ij, double *e_out) {
  double r = sqrt(r2);
  int clamped = r < 0.01;
  if (clamped) r = 0.01;
  double s = 1.0, w = 1.0, dw = 0.0; /* dw = dw/dr */
  if (shifted) {
    double t = r / 12.0;
    s = 1.0 - t * t;
    w = s * s;
    dw = 2.0 * s * (-2.0 * r / 144.0);
  }
  double p6 = pow6(x_ij / r);
  double lj = d_ij * (p6 * p6 - 2.0 * p6);
  double dlj = d_ij * (2.0 * p6 * (-6.0 * p6 / r) - 2.0 * (-6.0 * p6 / r)); /* d/dr */
  double el, del;
  if (dielectric == 1) {
    el = qqK / (r * r);
    del = -2.0 * qqK / (r * r * r);
  } else {
    el = qqK / r;
    del = -qqK / (r * r);
  }
  double e = lj + el;
  *e_out = w * e;
  if (clamped) return 0.0;
  double dEdr = dw * e + w * (dlj + del);
  return dEdr / r; /* dE/dd = (dE/dr) d / r */
}

/* the same pair term with every part taken by its absolute value:
 * *e_out = w (|el| + D p6^2 + 2 D p6) and the return value bounds |dE/dd| / r
 * by the same split of the derivative's parts */
static double pair_energy_grad_abs(int dielectric, int shifted, double r2, double qqK,
                                   double x_ij, double d_ij, double *e_out) {
  double r = sqrt(r2);
  int clamped = r < 0.01;
  if (clamped) r = 0.01;
  double w = 1.0, dw = 0.0;
  if (shifted) {
    double t = r / 12.0, s = 1.0 - t * t;
    w = s * s;
    dw = fabs(2.0 * s * (-2.0 * r / 144.0));
  }
  double p6 = pow6(x_ij / r);
  double lj = fabs(d_ij) * (p6 * p6 + 2.0 * p6);
  double dlj = fabs(d_ij) * (12.0 * p6 * p6 / r + 12.0 * p6 / r);
  double el, del;
  if (dielectric == 1) {
    el = fabs(qqK) / (r * r);
    del = 2.0 * fabs(qqK) / (r * r * r);
  } else {
    el = fabs(qqK) / r;
    del = fabs(qqK) / (r * r);
  }
  *e_out = w * (lj + el);
  if (clamped) return 0.0;
  return (dw * (lj + el) + w * (dlj + del)) / r;
}

/* analytic reverse-mode gradient; see uff_oracle.h */
double orc_grad_analytic(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                         const double *conf, int flags, double *grad, double *gxyz,
                         int *status) {
  int n = lig->m.n, nrb = lig->nrb;
  double K = orc_elec_weight();
  /* forward with snapshots of every stage of the torsion chain */
  double *snap = (double *)malloc(sizeof(double) * 3 * n * (nrb + 1) + 1);
  double *Zx = snap, *Zy = snap + n, *Zz = snap + 2 * n;
  memcpy(Zx, lig->m.x, sizeof(double) * n);
  memcpy(Zy, lig->m.y, sizeof(double) * n);
  memcpy(Zz, lig->m.z, sizeof(double) * n);
  for (int t = 0; t < nrb; ++t) {
    double *px = snap + 3 * n * t, *nx = snap + 3 * n * (t + 1);
    memcpy(nx, px, sizeof(double) * 3 * n);
    orc_rotate_bond(n, nx, nx + n, nx + 2 * n, lig->bond_lr[2 * t], lig->bond_lr[2 * t + 1],
                    lig->grp_atoms + lig->grp_off[t], lig->grp_off[t + 1] - lig->grp_off[t],
                    conf[6 + t]);
  }
  double *Y = snap + 3 * n * nrb;
  int st = too_long(n, Y, Y + n, Y + 2 * n) ? ORC_S_TOO_LONG : 0;
  double R[9], ctr[3] = {0, 0, 0};
  orc_rot_xyz(conf[3], conf[4], conf[5], R);
  if (flags & ORC_F_RECENTER) centroid(n, Y, Y + n, Y + 2 * n, ctr);
  double *X = (double *)malloc(sizeof(double) * 3 * n + 1);
  double *Yc = (double *)malloc(sizeof(double) * 3 * n + 1);
  double *G = (double *)calloc(3 * n + 1, sizeof(double));
  for (int i = 0; i < n; ++i) {
    double v[3] = {Y[i] - ctr[0], Y[n + i] - ctr[1], Y[2 * n + i] - ctr[2]}, w[3];
    Yc[3 * i] = v[0];
    Yc[3 * i + 1] = v[1];
    Yc[3 * i + 2] = v[2];
    matvec(R, v, w);
    for (int d = 0; d < 3; ++d) X[3 * i + d] = w[d] + conf[d];
  }
  /* energy and dE/dX */
  double E = 0.0;
  if (flags & ORC_F_INTER) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < prot->n; ++i) {
        double d[3] = {X[3 * j] - prot->x[i], X[3 * j + 1] - prot->y[i],
                       X[3 * j + 2] - prot->z[i]};
        double r2 = dot(d, d);
        if (ph->inter_form == 0 && !(r2 < 144.0)) continue;
        double x_ij, d_ij, e;
        orc_pair_params(ph, prot->anum[i], lig->m.anum[j], &x_ij, &d_ij);
        double g = pair_energy_grad(ph->dielectric, ph->inter_form == 0, r2,
                                    K * prot->q[i] * lig->m.q[j], x_ij, d_ij, &e);
        E += e;
        for (int k = 0; k < 3; ++k) G[3 * j + k] += g * d[k];
      }
  }
  if (flags & ORC_F_INTRA) {
    for (int i = 0; i < n - 1; ++i)
      for (int j = i + 1; j < n; ++j) {
        if (!lig->interacting[i * n + j]) continue;
        double d[3] = {X[3 * i] - X[3 * j], X[3 * i + 1] - X[3 * j + 1],
                       X[3 * i + 2] - X[3 * j + 2]};
        double r2 = dot(d, d);
        int shifted = ph->intra_form == 1;
        if (shifted && !(orc_non_zero_dist(sqrt(r2)) < 12.0)) continue;
        double x_ij, d_ij, e;
        orc_pair_params(ph, lig->m.anum[i], lig->m.anum[j], &x_ij, &d_ij);
        double g = pair_energy_grad(ph->dielectric, shifted, r2, K * lig->m.q[i] * lig->m.q[j],
                                    x_ij, d_ij, &e);
        E += e;
        for (int k = 0; k < 3; ++k) {
          G[3 * i + k] += g * d[k];
          G[3 * j + k] -= g * d[k];
        }
      }
  }
  if (gxyz) memcpy(gxyz, G, sizeof(double) * 3 * n);
  /* rigid part */
  double dA[9], dB[9], dG[9], M[9] = {0};
  rot_xyz_derivs(conf[3], conf[4], conf[5], dA, dB, dG);
  grad[0] = grad[1] = grad[2] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      grad[k] += G[3 * i + k];
      for (int l = 0; l < 3; ++l) M[3 * k + l] += G[3 * i + k] * Yc[3 * i + l];
    }
  grad[3] = grad[4] = grad[5] = 0.0;
  for (int e = 0; e < 9; ++e) {
    grad[3] += M[e] * dA[e];
    grad[4] += M[e] * dB[e];
    grad[5] += M[e] * dG[e];
  }
  /* adjoint of Y */
  double *A = (double *)malloc(sizeof(double) * 3 * n + 1);
  double mean[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    matTvec(R, G + 3 * i, A + 3 * i);
    for (int k = 0; k < 3; ++k) mean[k] += A[3 * i + k];
  }
  if (flags & ORC_F_RECENTER)
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) A[3 * i + k] -= mean[k] / n;
  /* reverse through the torsions */
  for (int t = nrb - 1; t >= 0; --t) {
    const double *pre = snap + 3 * n * t, *post = snap + 3 * n * (t + 1);
    int left = lig->bond_lr[2 * t], right = lig->bond_lr[2 * t + 1];
    double c[3], a[3], u[3], alen, Rt[9];
    bond_axis(pre, pre + n, pre + 2 * n, left, right, c, a, u, &alen);
    double th = conf[6 + t], ct = cos(th), stt = sin(th);
    orc_rot_axis_angle(u, th, Rt);
    double dth = 0.0, dU[3] = {0, 0, 0}, dC[3] = {0, 0, 0};
    for (int k = lig->grp_off[t]; k < lig->grp_off[t + 1]; ++k) {
      int i = lig->grp_atoms[k];
      double vp[3] = {post[i] - c[0], post[n + i] - c[1], post[2 * n + i] - c[2]};
      double v[3] = {pre[i] - c[0], pre[n + i] - c[1], pre[2 * n + i] - c[2]};
      double *Ai = A + 3 * i, uxv[3], vxA[3], RtA[3];
      cross(u, vp, uxv);
      dth += dot(Ai, uxv);
      cross(v, Ai, vxA);
      double uv = dot(u, v), Au = dot(Ai, u);
      for (int d = 0; d < 3; ++d) dU[d] += stt * vxA[d] + (1.0 - ct) * (uv * Ai[d] + Au * v[d]);
      matTvec(Rt, Ai, RtA);
      for (int d = 0; d < 3; ++d) {
        dC[d] += Ai[d] - RtA[d];
        Ai[d] = RtA[d];
      }
    }
    grad[6 + t] = dth;
    double uu = dot(u, dU), da[3];
    for (int d = 0; d < 3; ++d) da[d] = (dU[d] - u[d] * uu) / alen;
    for (int d = 0; d < 3; ++d) {
      A[3 * right + d] += da[d] + dC[d];
      A[3 * left + d] -= da[d];
    }
  }
  if (!isfinite(E)) st |= ORC_S_NONFINITE;
  if (status) *status = st;
  free(A);
  free(G);
  free(Yc);
  free(X);
  free(snap);
  return E;
}

/* ---- condition scales of the energy and of each gradient component --------
 * The same forward pass and reverse pass as orc_grad_analytic, with every sum
 * of terms replaced by the sum of their absolute values and every product by
 * the product of absolute values (|a x b| by the componentwise bound
 * |a_y||b_z| + |a_z||b_y|, a matrix by its entrywise absolute value), and each
 * pair term split into its parts (elec, the two LJ powers, the switch).  The
 * energy scale is S = sum over pairs of w (|elec| + D (x/r)^12 + 2 D (x/r)^6);
 * grad_abs[k] bounds the sum of |terms| that the analytic gradient adds into
 * component k.  A floating-point evaluation of the same sums with unit
 * round-off u is accurate to about u * scale, whatever the cancellation. */
static void abs3(const double a[3], double o[3]) {
  o[0] = fabs(a[0]);
  o[1] = fabs(a[1]);
  o[2] = fabs(a[2]);
}
static void cross_abs(const double a[3], const double b[3], double c[3]) {
  c[0] = fabs(a[1] * b[2]) + fabs(a[2] * b[1]);
  c[1] = fabs(a[2] * b[0]) + fabs(a[0] * b[2]);
  c[2] = fabs(a[0] * b[1]) + fabs(a[1] * b[0]);
}
static double dot_abs(const double a[3], const double b[3]) {
  return fabs(a[0] * b[0]) + fabs(a[1] * b[1]) + fabs(a[2] * b[2]);
}

double orc_grad_scale(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                      const double *conf, int flags, double *grad_abs) {
  int n = lig->m.n, nrb = lig->nrb;
  double K = orc_elec_weight();
  double *snap = (double *)malloc(sizeof(double) * 3 * n * (nrb + 1) + 1);
  memcpy(snap, lig->m.x, sizeof(double) * n);
  memcpy(snap + n, lig->m.y, sizeof(double) * n);
  memcpy(snap + 2 * n, lig->m.z, sizeof(double) * n);
  for (int t = 0; t < nrb; ++t) {
    double *px = snap + 3 * n * t, *nx = snap + 3 * n * (t + 1);
    memcpy(nx, px, sizeof(double) * 3 * n);
    orc_rotate_bond(n, nx, nx + n, nx + 2 * n, lig->bond_lr[2 * t], lig->bond_lr[2 * t + 1],
                    lig->grp_atoms + lig->grp_off[t], lig->grp_off[t + 1] - lig->grp_off[t],
                    conf[6 + t]);
  }
  double *Y = snap + 3 * n * nrb;
  double R[9], Ra[9], ctr[3] = {0, 0, 0};
  orc_rot_xyz(conf[3], conf[4], conf[5], R);
  for (int e = 0; e < 9; ++e) Ra[e] = fabs(R[e]);
  if (flags & ORC_F_RECENTER) centroid(n, Y, Y + n, Y + 2 * n, ctr);
  double *X = (double *)malloc(sizeof(double) * 3 * n + 1);
  double *Yc = (double *)malloc(sizeof(double) * 3 * n + 1);
  double *G = (double *)calloc(3 * n + 1, sizeof(double));
  for (int i = 0; i < n; ++i) {
    double v[3] = {Y[i] - ctr[0], Y[n + i] - ctr[1], Y[2 * n + i] - ctr[2]}, w[3];
    for (int d = 0; d < 3; ++d) Yc[3 * i + d] = fabs(v[d]);
    matvec(R, v, w);
    for (int d = 0; d < 3; ++d) X[3 * i + d] = w[d] + conf[d];
  }
  double S = 0.0;
  if (flags & ORC_F_INTER) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < prot->n; ++i) {
        double d[3] = {X[3 * j] - prot->x[i], X[3 * j + 1] - prot->y[i],
                       X[3 * j + 2] - prot->z[i]};
        double r2 = dot(d, d);
        if (ph->inter_form == 0 && !(r2 < 144.0)) continue;
        double x_ij, d_ij, e;
        orc_pair_params(ph, prot->anum[i], lig->m.anum[j], &x_ij, &d_ij);
        double g = pair_energy_grad_abs(ph->dielectric, ph->inter_form == 0, r2,
                                        K * prot->q[i] * lig->m.q[j], x_ij, d_ij, &e);
        S += e;
        for (int k = 0; k < 3; ++k) G[3 * j + k] += g * fabs(d[k]);
      }
  }
  if (flags & ORC_F_INTRA) {
    for (int i = 0; i < n - 1; ++i)
      for (int j = i + 1; j < n; ++j) {
        if (!lig->interacting[i * n + j]) continue;
        double d[3] = {X[3 * i] - X[3 * j], X[3 * i + 1] - X[3 * j + 1],
                       X[3 * i + 2] - X[3 * j + 2]};
        double r2 = dot(d, d);
        int shifted = ph->intra_form == 1;
        if (shifted && !(orc_non_zero_dist(sqrt(r2)) < 12.0)) continue;
        double x_ij, d_ij, e;
        orc_pair_params(ph, lig->m.anum[i], lig->m.anum[j], &x_ij, &d_ij);
        double g = pair_energy_grad_abs(ph->dielectric, shifted, r2,
                                        K * lig->m.q[i] * lig->m.q[j], x_ij, d_ij, &e);
        S += e;
        for (int k = 0; k < 3; ++k) {
          G[3 * i + k] += g * fabs(d[k]);
          G[3 * j + k] += g * fabs(d[k]);
        }
      }
  }
  double dA[9], dB[9], dG[9], M[9] = {0};
  rot_xyz_derivs(conf[3], conf[4], conf[5], dA, dB, dG);
  grad_abs[0] = grad_abs[1] = grad_abs[2] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      grad_abs[k] += G[3 * i + k];
      for (int l = 0; l < 3; ++l) M[3 * k + l] += G[3 * i + k] * Yc[3 * i + l];
    }
  grad_abs[3] = grad_abs[4] = grad_abs[5] = 0.0;
  for (int e = 0; e < 9; ++e) {
    grad_abs[3] += M[e] * fabs(dA[e]);
    grad_abs[4] += M[e] * fabs(dB[e]);
    grad_abs[5] += M[e] * fabs(dG[e]);
  }
  double *A = (double *)malloc(sizeof(double) * 3 * n + 1);
  double mean[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    matTvec(Ra, G + 3 * i, A + 3 * i);
    for (int k = 0; k < 3; ++k) mean[k] += A[3 * i + k];
  }
  if (flags & ORC_F_RECENTER)
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) A[3 * i + k] += mean[k] / n;
  for (int t = nrb - 1; t >= 0; --t) {
    const double *pre = snap + 3 * n * t, *post = snap + 3 * n * (t + 1);
    int left = lig->bond_lr[2 * t], right = lig->bond_lr[2 * t + 1];
    double c[3], a[3], u[3], alen, Rt[9], ua[3];
    bond_axis(pre, pre + n, pre + 2 * n, left, right, c, a, u, &alen);
    double th = conf[6 + t], ct = fabs(1.0 - cos(th)), stt = fabs(sin(th));
    orc_rot_axis_angle(u, th, Rt);
    for (int e = 0; e < 9; ++e) Rt[e] = fabs(Rt[e]);
    abs3(u, ua);
    double dth = 0.0, dU[3] = {0, 0, 0}, dC[3] = {0, 0, 0};
    for (int k = lig->grp_off[t]; k < lig->grp_off[t + 1]; ++k) {
      int i = lig->grp_atoms[k];
      double vp[3] = {post[i] - c[0], post[n + i] - c[1], post[2 * n + i] - c[2]};
      double v[3] = {pre[i] - c[0], pre[n + i] - c[1], pre[2 * n + i] - c[2]}, va[3];
      double *Ai = A + 3 * i, uxv[3], vxA[3], RtA[3];
      abs3(v, va);
      cross_abs(u, vp, uxv);
      dth += dot_abs(Ai, uxv);
      cross_abs(v, Ai, vxA);
      double uv = dot_abs(u, v), Au = dot_abs(Ai, u);
      for (int d = 0; d < 3; ++d) dU[d] += stt * vxA[d] + ct * (uv * Ai[d] + Au * va[d]);
      matTvec(Rt, Ai, RtA);
      for (int d = 0; d < 3; ++d) {
        dC[d] += Ai[d] + RtA[d];
        Ai[d] = RtA[d];
      }
    }
    grad_abs[6 + t] = dth;
    double uu = dot_abs(ua, dU);
    for (int d = 0; d < 3; ++d) {
      double da = (dU[d] + ua[d] * uu) / alen;
      A[3 * right + d] += da + dC[d];
      A[3 * left + d] += da;
    }
  }
  free(A);
  free(G);
  free(Yc);
  free(X);
  free(snap);
  return S;
}

/* ---- batch over poses on host threads ------------------------------------ */
typedef struct {
  const orc_physics *ph;
  const orc_mol *prot;
  const orc_cells *cells;
  const orc_ligand *lig;
  const float *dofs;
  int flags, mode, b0, b1, nd;
  const double *eps;
  double *E, *grad;
  int *status;
} batch_job;

static void *batch_worker(void *arg) {
  batch_job *j = (batch_job *)arg;
  double conf[64 + 6];
  for (int b = j->b0; b < j->b1; ++b) {
    for (int k = 0; k < j->nd; ++k) conf[k] = (double)j->dofs[(size_t)b * j->nd + k];
    int st = 0;
    double *g = j->grad ? j->grad + (size_t)b * j->nd : NULL;
    if (j->mode == 1 && g) {
      j->E[b] = orc_grad_analytic(j->ph, j->prot, j->lig, conf, j->flags, g, NULL, &st);
    } else if (j->mode == 3 && g) {
      j->E[b] = orc_grad_scale(j->ph, j->prot, j->lig, conf, j->flags, g);
    } else {
      j->E[b] = orc_score_conf(j->ph, j->prot, j->cells, j->lig, conf, j->flags, &st);
      if (j->mode == 2 && g) orc_grad_fd(j->ph, j->prot, j->cells, j->lig, conf, j->flags, j->eps, g);
    }
    if (j->status) j->status[b] = st;
  }
  return NULL;
}

void orc_score_batch(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig, int B,
                     const float *dofs, int flags, int mode, const double *eps, int use_cells,
                     int nthreads, double *E, double *grad, int *status) {
  orc_cells *cells = (use_cells && ph->inter_form == 0) ? orc_cells_build(prot) : NULL;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > B) nthreads = B > 0 ? B : 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  batch_job *jobs = (batch_job *)malloc(sizeof(batch_job) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    batch_job j = {ph, prot, cells, lig, dofs, flags, mode,
                   (int)((long)B * t / nthreads), (int)((long)B * (t + 1) / nthreads),
                   6 + lig->nrb, eps, E, grad, status};
    jobs[t] = j;
    if (nthreads == 1)
      batch_worker(&jobs[t]);
    else
      pthread_create(&th[t], NULL, batch_worker, &jobs[t]);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  orc_cells_free(cells);
}

/* ---- counter-based RNG of the Monte Carlo chains ---------------------------
 * Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC 2011): ten rounds of two 32x32->64
 * multiplications by 0xD2511F53 and 0xCD9E8D57, the key bumped by the Weyl
 * constants 0x9E3779B9 and 0xBB67AE85 between rounds.  The reference draws from
 * OCaml's Random.State (src/lds.ml:931-934, src/move.ml:14-54); a counter-based
 * generator keyed per chain replaces it so that chains are independent and
 * reproducible in parallel. */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* ---- precomputed grids and their trilinear interpolation -------------------
 * orc_grid_point: Mol.ene_inter_UFF_shifted_grid (src/mol.ml:964-989) at one
 * point for single-atom "ligands" of (anum, charge) types, capped at max_E as
 * Lds.pre_calculate_FF_components_grid does (src/lds.ml:452-469):
 *   E_l(p) = min(max_E, K sum_i w q_i q_l / r + sum_i w D_il (p6^2 - 2 p6)),
 * r = max(|p - r_i|, 0.01), w = shift_12A(r), over the protein atoms within
 * 12 A.  The dielectric switch of ph selects q/r (eps 4, the reference) or
 * q/r^2 (eps 4r). */
void orc_grid_point(const orc_physics *ph, const orc_mol *prot, const double p[3], int ntypes,
                    const int *type_anum, const double *type_q, double max_E, double *out) {
  for (int l = 0; l < ntypes; ++l) {
    double se = 0.0, sv = 0.0;
    for (int i = 0; i < prot->n; ++i) {
      const double dx = p[0] - prot->x[i], dy = p[1] - prot->y[i], dz = p[2] - prot->z[i];
      const double d2 = dx * dx + dy * dy + dz * dz;
      if (!(d2 < 144.0)) continue;
      const double r = orc_non_zero_dist(sqrt(d2));
      const double w = orc_shift_12A(r);
      double x_ij, d_ij;
      orc_pair_params(ph, type_anum[l], prot->anum[i], &x_ij, &d_ij);
      const double p1 = x_ij / r, p6 = p1 * p1 * p1 * p1 * p1 * p1;
      se += w * (prot->q[i] * type_q[l]) / (ph->dielectric ? r * r : r);
      sv += w * (d_ij * ((-2.0 * p6) + (p6 * p6)));
    }
    const double e = orc_elec_weight() * se + sv;
    out[l] = e < max_E ? e : max_E;
  }
}

/* G3D.trilin (src/G3D.ml:97-157) on a lattice with its lowest point at the
 * origin (x = i step), values x-fastest: v[i + j nx + k nx ny] (float32, as the
 * reference's .ba1 files).  Returns 0 and sets *off when a corner falls off the
 * lattice (the reference does not check). */
double orc_trilin(double step, int nx, int ny, int nz, const float *v, const double p[3],
                  int *off) {
  const double inv = 1.0 / step;
  const double ux = p[0] * inv, uy = p[1] * inv, uz = p[2] * inv;
  /* the high corner (int) u + 1 is on the lattice iff 0 <= u < n - 1 (tested
   * before the conversion, which is undefined for huge u) */
  if (!(ux >= 0 && uy >= 0 && uz >= 0 && ux < nx - 1 && uy < ny - 1 && uz < nz - 1)) {
    if (off) *off = 1;
    return 0.0;
  }
  const int i0 = (int)ux, j0 = (int)uy, k0 = (int)uz;
  const int i1 = i0 + 1, j1 = j0 + 1, k1 = k0 + 1;
  const long j0x = (long)j0 * nx, j1x = (long)j1 * nx, k0xy = (long)k0 * nx * ny,
             k1xy = (long)k1 * nx * ny;
  const double wlx = (p[0] - i0 * step) * inv, wly = (p[1] - j0 * step) * inv,
               wlz = (p[2] - k0 * step) * inv;
  const double whx = 1.0 - wlx, why = 1.0 - wly, whz = 1.0 - wlz;
  return v[i0 + j0x + k0xy] * (whx * why * whz) + v[i1 + j0x + k0xy] * (wlx * why * whz) +
         v[i1 + j1x + k0xy] * (wlx * wly * whz) + v[i0 + j1x + k0xy] * (whx * wly * whz) +
         v[i0 + j0x + k1xy] * (whx * why * wlz) + v[i1 + j0x + k1xy] * (wlx * why * wlz) +
         v[i1 + j1x + k1xy] * (wlx * wly * wlz) + v[i0 + j1x + k1xy] * (whx * wly * wlz);
}

/* Mol.ene_inter_UFF_interp (src/mol.ml:1010-1020): sum over the ligand atoms of
 * the trilinear value of the atom type's grid at the atom (coordinates in the
 * lattice frame). */
double orc_ene_inter_interp(double step, int nx, int ny, int nz, const float *grids, int n,
                            const double *x, const double *y, const double *z, const int *type,
                            int *off) {
  double e = 0.0;
  const size_t per = (size_t)nx * ny * nz;
  for (int j = 0; j < n; ++j) {
    const double p[3] = {x[j], y[j], z[j]};
    e += orc_trilin(step, nx, ny, nz, grids + per * type[j], p, off);
  }
  return e;
}

/* orc_grid_point at n points (pts[n][3]) into out[n][ntypes] through the cell
 * list (scale, if not NULL: the sum of |pair terms| of each value), with the factorisation of Mol.ene_inter_UFF_shifted_grid
 * (src/mol.ml:964-989): the point's neighbours within 12 A once, then every
 * type; pair parameters looked up per (type, protein element).  nthreads
 * POSIX threads over the points. */
typedef struct {
  const orc_physics *ph;
  const orc_cells *cells;
  const double *pts;
  int p0, p1, ntypes;
  const double *type_q;
  const double *xt, *dt; /* [ntypes][128] x_ij, D_ij by protein atomic number */
  double max_E;
  double *out, *scale;
} grid_job;

static void *grid_worker(void *arg) {
  grid_job *J = (grid_job *)arg;
  const orc_cells *c = J->cells;
  const orc_mol *prot = &c->prot;
  const int nt = J->ntypes;
  double *se = (double *)malloc(sizeof(double) * 3 * (size_t)nt);
  double *sv = se + nt, *sa = sv + nt;
  for (int k = J->p0; k < J->p1; ++k) {
    const double *p = J->pts + 3 * (size_t)k;
    for (int l = 0; l < nt; ++l) se[l] = sv[l] = sa[l] = 0.0;
    const int cx = (int)floor((p[0] - c->lo[0]) / CUTOFF);
    const int cy = (int)floor((p[1] - c->lo[1]) / CUTOFF);
    const int cz = (int)floor((p[2] - c->lo[2]) / CUTOFF);
    for (int gz = cz - 1; gz <= cz + 1; ++gz) {
      if (gz < 0 || gz >= c->dim[2]) continue;
      for (int gy = cy - 1; gy <= cy + 1; ++gy) {
        if (gy < 0 || gy >= c->dim[1]) continue;
        for (int gx = cx - 1; gx <= cx + 1; ++gx) {
          if (gx < 0 || gx >= c->dim[0]) continue;
          const int cell = (gz * c->dim[1] + gy) * c->dim[0] + gx;
          for (int m = c->start[cell]; m < c->start[cell + 1]; ++m) {
            const int i = c->idx[m];
            const double dx = p[0] - prot->x[i], dy = p[1] - prot->y[i], dz = p[2] - prot->z[i];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 < 144.0)) continue;
            const double r = orc_non_zero_dist(sqrt(d2));
            const double w = orc_shift_12A(r);
            const double qr = prot->q[i] / (J->ph->dielectric ? r * r : r);
            const int an = prot->anum[i] & 127;
            for (int l = 0; l < nt; ++l) {
              const double p1 = J->xt[l * 128 + an] / r, p2 = p1 * p1, p6 = p2 * p2 * p2;
              const double el = w * (qr * J->type_q[l]);
              const double vd = w * (J->dt[l * 128 + an] * ((-2.0 * p6) + (p6 * p6)));
              se[l] += el;
              sv[l] += vd;
              if (J->scale) sa[l] += orc_elec_weight() * fabs(el) + fabs(vd);
            }
          }
        }
      }
    }
    for (int l = 0; l < nt; ++l) {
      const double e = orc_elec_weight() * se[l] + sv[l];
      J->out[(size_t)k * nt + l] = e < J->max_E ? e : J->max_E;
      if (J->scale) J->scale[(size_t)k * nt + l] = sa[l];
    }
  }
  free(se);
  return NULL;
}

void orc_grid_points(const orc_physics *ph, const orc_mol *prot, int n, const double *pts,
                     int ntypes, const int *type_anum, const double *type_q, double max_E,
                     int nthreads, double *out, double *scale) {
  orc_cells *cells = orc_cells_build(prot);
  double *xt = (double *)calloc((size_t)ntypes * 256, sizeof(double));
  double *dt = xt + (size_t)ntypes * 128;
  for (int l = 0; l < ntypes; ++l)
    for (int i = 0; i < prot->n; ++i) {
      const int an = prot->anum[i] & 127;
      orc_pair_params(ph, type_anum[l], prot->anum[i], &xt[l * 128 + an], &dt[l * 128 + an]);
    }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > n) nthreads = n > 0 ? n : 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  grid_job *jobs = (grid_job *)malloc(sizeof(grid_job) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    grid_job J = {ph, cells, pts, (int)((long)n * t / nthreads),
                  (int)((long)n * (t + 1) / nthreads), ntypes, type_q, xt, dt, max_E, out, scale};
    jobs[t] = J;
    if (nthreads == 1)
      grid_worker(&jobs[t]);
    else
      pthread_create(&th[t], NULL, grid_worker, &jobs[t]);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  free(xt);
  orc_cells_free(cells);
}

/* ---- lattice masks, clash tests, SO(3) samples, exhaustive docking,
 *      desolvation ------------------------------------------------------------
 * The lattice of the grids: point (i, j, k) at o + step (i, j, k), index
 * i + j nx + k nx ny (src/grid.ml).  Masks are one byte per point. */

#define ORC_PI 3.14159265358979323846

/* Ptable.vdW_radii (src/ptable.ml:41-53); NaN for other elements */
double orc_vdw_radius(int anum) {
  switch (anum) {
    case 1: return 1.2;
    case 6: return 1.7;
    case 7: return 1.6;
    case 8: return 1.55;
    case 9: return 1.5;
    case 12: return 2.2;
    case 15: return 1.95;
    case 16: return 1.8;
    case 17: return 1.8;
    case 35: return 1.9;
    case 53: return 2.1;
    default: return NAN;
  }
}

/* Ptable.vdW_clash_params2 (src/ptable.ml:62-80): (0.8 (r_i + r_j))^2 */
double orc_clash2(int a1, int a2) {
  const double x = 0.8 * (orc_vdw_radius(a1) + orc_vdw_radius(a2));
  return x * x;
}

/* Lds.atom_bitmask_set (src/lds.ml:149-169): the points of the cube of
 * ceil(radius / step) cells about the atom's cell (Grid.coord_of_point:
 * truncation toward zero) within radius are set to b; points off the lattice
 * are skipped (the reference has the simulation box's margin for them). */
void orc_atom_bitmask_set(const orc_lattice *g, const double p[3], double radius, uint8_t b,
                          uint8_t *mask) {
  const int ci = (int)((p[0] - g->o[0]) / g->step), cj = (int)((p[1] - g->o[1]) / g->step),
            ck = (int)((p[2] - g->o[2]) / g->step);
  const int rs = (int)ceil(radius / g->step);
  const double r2 = radius * radius;
  for (int i = ci - rs; i <= ci + rs; ++i) {
    if (i < 0 || i >= g->nx) continue;
    const double x = g->o[0] + g->step * i;
    for (int j = cj - rs; j <= cj + rs; ++j) {
      if (j < 0 || j >= g->ny) continue;
      const double y = g->o[1] + g->step * j;
      for (int k = ck - rs; k <= ck + rs; ++k) {
        if (k < 0 || k >= g->nz) continue;
        const double z = g->o[2] + g->step * k;
        const double dx = p[0] - x, dy = p[1] - y, dz = p[2] - z;
        if (dx * dx + dy * dy + dz * dz < r2)
          mask[i + (size_t)j * g->nx + (size_t)k * g->nx * g->ny] = b;
      }
    }
  }
}

/* Lds.vdW_volume (src/lds.ml:187-196) and Lds.first_solvent_shell
 * (src/lds.ml:172-184): every point within r_i of an atom; every point within
 * r_i + r_w of an atom and within r_j of none.  Either output may be NULL. */
void orc_masks(const orc_lattice *g, int n, const double *x, const double *y, const double *z,
               const double *radius, double r_w, uint8_t *vdw, uint8_t *shell) {
  const size_t np = (size_t)g->nx * g->ny * g->nz;
  if (vdw) {
    memset(vdw, 0, np);
    for (int a = 0; a < n; ++a) {
      const double p[3] = {x[a], y[a], z[a]};
      orc_atom_bitmask_set(g, p, radius[a], 1, vdw);
    }
  }
  if (shell) {
    memset(shell, 0, np);
    for (int a = 0; a < n; ++a) {
      const double p[3] = {x[a], y[a], z[a]};
      orc_atom_bitmask_set(g, p, radius[a] + r_w, 1, shell);
    }
    for (int a = 0; a < n; ++a) {
      const double p[3] = {x[a], y[a], z[a]};
      orc_atom_bitmask_set(g, p, radius[a], 0, shell);
    }
  }
}

/* G3D.vdW_clash_OR / vdW_clash_AND (src/G3D.ml:159-213): the eight corners of
 * p's cell; a corner off the lattice counts as not set (the reference reads out
 * of bounds there). */
static int corner_bits(const orc_lattice *g, const uint8_t *mask, const double p[3], int *all) {
  const double u = (p[0] - g->o[0]) / g->step, v = (p[1] - g->o[1]) / g->step,
               w = (p[2] - g->o[2]) / g->step;
  int any = 0, every = 1;
  const int i0 = (int)u, j0 = (int)v, k0 = (int)w;
  for (int c = 0; c < 8; ++c) {
    const int i = i0 + (c & 1), j = j0 + ((c >> 1) & 1), k = k0 + (c >> 2);
    int bit = 0;
    if (u > -1.0 && v > -1.0 && w > -1.0 && i >= 0 && j >= 0 && k >= 0 && i < g->nx &&
        j < g->ny && k < g->nz && u < 2e9 && v < 2e9 && w < 2e9)
      bit = mask[i + (size_t)j * g->nx + (size_t)k * g->nx * g->ny] != 0;
    any |= bit;
    every &= bit;
  }
  *all = every;
  return any;
}

int orc_clash_or(const orc_lattice *g, const uint8_t *mask, const double p[3]) {
  int all;
  return corner_bits(g, mask, p, &all);
}

int orc_clash_and(const orc_lattice *g, const uint8_t *mask, const double p[3]) {
  int all;
  corner_bits(g, mask, p, &all);
  return all;
}

/* Mol.protein_ligand_clash (src/mol.ml:1195-1207): any atom's cell touches the
 * protein's vdW volume */
int orc_protein_ligand_clash(const orc_lattice *g, const uint8_t *vdw, int n, const double *x,
                             const double *y, const double *z) {
  for (int a = 0; a < n; ++a) {
    const double p[3] = {x[a], y[a], z[a]};
    if (orc_clash_or(g, vdw, p)) return 1;
  }
  return 0;
}

/* Mol.is_ligand_center_vdW_occuppied (src/mol.ml:1209-1219) */
int orc_center_occupied(int n, const double *x, const double *y, const double *z,
                        const double *radius) {
  double c[3] = {0, 0, 0};
  for (int a = 0; a < n; ++a) {
    c[0] += x[a];
    c[1] += y[a];
    c[2] += z[a];
  }
  for (int d = 0; d < 3; ++d) c[d] /= n;
  for (int a = 0; a < n; ++a) {
    const double dx = c[0] - x[a], dy = c[1] - y[a], dz = c[2] - z[a];
    if (sqrt(dx * dx + dy * dy + dz * dz) < radius[a]) return 1;
  }
  return 0;
}

/* Mol.heavy_atom_clash (src/mol.ml:1170-1190): a ligand heavy atom (anum > 1)
 * closer than 0.8 (r_i + r_j) to a protein heavy atom.  The reference
 * gathers the candidates with a BST query of radius 2 Ptable.vdW_max, whose
 * value is the intended 4.4 A here (every closer pair is a candidate). */
int orc_heavy_atom_clash(const orc_mol *prot, int n, const double *x, const double *y,
                         const double *z, const int *anum) {
  for (int a = 0; a < n; ++a) {
    if (anum[a] <= 1) continue;
    for (int i = 0; i < prot->n; ++i) {
      if (prot->anum[i] <= 1) continue;
      const double dx = x[a] - prot->x[i], dy = y[a] - prot->y[i], dz = z[a] - prot->z[i];
      if (dx * dx + dy * dy + dz * dz < orc_clash2(anum[a], prot->anum[i])) return 1;
    }
  }
  return 0;
}

/* Mol.ligand_atoms_clash_fast (src/mol.ml:1077-1088): a pair at topological
 * distance >= 3 closer than 0.8 (r_i + r_j) */
int orc_intra_clash(int n, const double *x, const double *y, const double *z, const int *anum,
                    const uint8_t *interacting) {
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      if (!interacting[(size_t)i * n + j]) continue;
      const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
      if (dx * dx + dy * dy + dz * dz < orc_clash2(anum[i], anum[j])) return 1;
    }
  return 0;
}

/* SO3.super_fibonacci and SO3.rotations (src/SO3.ml:18-46, after Alexa, CVPR
 * 2022, Algorithm 1): sample i of n as the quaternion
 * (w, x, y, z) = (sqrt(t) sin(a), sqrt(t) cos(a), sqrt(1-t) sin(b), sqrt(1-t) cos(b)),
 * s = i + 1/2, t = s / n, a = 2 pi s / sqrt(2), b = 2 pi s / psi, then the
 * rotation of its axis and angle (Quat.to_axis_angle, Rot.of_axis_angle). */
void orc_so3_rotation(int n, int i, double R[9]) {
  const double phi = sqrt(2.0), psi = 1.533751168755204288118041;
  const double s = (double)i + 0.5, t = s / (double)n, d = 2.0 * ORC_PI * s;
  const double cr = sqrt(t), cR = sqrt(1.0 - t), al = d / phi, be = d / psi;
  const double w = cr * sin(al), x = cr * cos(al), y = cR * sin(be), z = cR * cos(be);
  const double mag = sqrt(x * x + y * y + z * z);
  const double u[3] = {x / mag, y / mag, z / mag};
  orc_rot_axis_angle(u, 2.0 * atan2(mag, w), R);
}

/* Lds.exhaustive_rigid_ligand_docking (src/lds.ml:1040-1114), every score:
 * positions on the lattice Grid.from_box(trans_step) of the ROI's bounding
 * cube (x_min + i step, ceil(2 r / step) + 1 points per axis), rotations
 * R_r (nrot); score[(pos index) nrot + r] = const_intra + the interpolated
 * inter energy of R_r x + pos, or +inf when pos is outside the ROI, when the
 * ligand's centre is vdW-occupied and all eight corners of pos's cell are in
 * the protein's vdW volume, or when the posed ligand clashes with it (any
 * corner).  Returns the position lattice's points per axis in dims. */
void orc_dock_scores(const orc_lattice *g, const float *grids, const uint8_t *vdw,
                     const orc_mol *lig, const int *lig_type, const double *lig_radius,
                     const double roi_c[3], double roi_r, double trans_step, int nrot,
                     const double *R, double const_intra, int dims[3], double *scores) {
  const int n = lig->n;
  const int center_occ = orc_center_occupied(n, lig->x, lig->y, lig->z, lig_radius);
  const int dim = (int)ceil(2.0 * roi_r / trans_step) + 1;
  dims[0] = dims[1] = dims[2] = dim;
  double *xs = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  double *ys = xs + n, *zs = ys + n;
  for (int k = 0; k < dim; ++k)
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) {
        const double pos[3] = {roi_c[0] - roi_r + trans_step * i, roi_c[1] - roi_r + trans_step * j,
                               roi_c[2] - roi_r + trans_step * k};
        const size_t pidx = (size_t)i + (size_t)j * dim + (size_t)k * dim * dim;
        const double dx = pos[0] - roi_c[0], dy = pos[1] - roi_c[1], dz = pos[2] - roi_c[2];
        const int skip = !(dx * dx + dy * dy + dz * dz < roi_r * roi_r) ||
                         (center_occ && orc_clash_and(g, vdw, pos));
        for (int r = 0; r < nrot; ++r) {
          double *out = scores + pidx * nrot + r;
          *out = INFINITY;
          if (skip) continue;
          const double *M = R + 9 * (size_t)r;
          for (int a = 0; a < n; ++a) {
            xs[a] = M[0] * lig->x[a] + M[1] * lig->y[a] + M[2] * lig->z[a] + pos[0];
            ys[a] = M[3] * lig->x[a] + M[4] * lig->y[a] + M[5] * lig->z[a] + pos[1];
            zs[a] = M[6] * lig->x[a] + M[7] * lig->y[a] + M[8] * lig->z[a] + pos[2];
          }
          if (orc_protein_ligand_clash(g, vdw, n, xs, ys, zs)) continue;
          double e = 0.0;
          const size_t per = (size_t)g->nx * g->ny * g->nz;
          int off = 0;
          for (int a = 0; a < n; ++a) {
            const double p[3] = {xs[a] - g->o[0], ys[a] - g->o[1], zs[a] - g->o[2]};
            e += orc_trilin(g->step, g->nx, g->ny, g->nz, grids + per * lig_type[a], p, &off);
          }
          *out = const_intra + e;
        }
      }
  free(xs);
}

/* Lds.protein_desolv (src/lds.ml:204-233): for every point of the protein's
 * solvent shell inside the ROI, C vol sum_j (q_j / d^2)^2 over the protein atoms
 * within 12 A, C = (1/eps_prot - 1/eps_water) / (8 pi) (src/const.ml:31); 0
 * elsewhere. */
double orc_desolv_constant(void) { return (1.0 / 4.0 - 1.0 / 78.5) / (8.0 * ORC_PI); }

void orc_protein_desolv(const orc_lattice *g, const orc_mol *prot, const uint8_t *shell,
                        const double roi_c[3], double roi_r, double *out) {
  const double vol = g->step * g->step * g->step;
  for (int k = 0; k < g->nz; ++k)
    for (int j = 0; j < g->ny; ++j)
      for (int i = 0; i < g->nx; ++i) {
        const size_t idx = i + (size_t)j * g->nx + (size_t)k * g->nx * g->ny;
        out[idx] = 0.0;
        if (!shell[idx]) continue;
        const double p[3] = {g->o[0] + g->step * i, g->o[1] + g->step * j, g->o[2] + g->step * k};
        const double rx = p[0] - roi_c[0], ry = p[1] - roi_c[1], rz = p[2] - roi_c[2];
        if (!(rx * rx + ry * ry + rz * rz < roi_r * roi_r)) continue;
        double s = 0.0;
        for (int a = 0; a < prot->n; ++a) {
          const double dx = p[0] - prot->x[a], dy = p[1] - prot->y[a], dz = p[2] - prot->z[a];
          const double d2 = dx * dx + dy * dy + dz * dz;
          if (!(d2 < 144.0)) continue;
          const double v = prot->q[a] / d2;
          s += v * v;
        }
        out[idx] = orc_desolv_constant() * (vol * s);
      }
}

/* Lds.desolvation_penalty (src/lds.ml:236-267): the points of both solvent
 * shells (the protein's and this ligand pose's); out[0] = the protein's
 * contributions summed over them, out[1] = C vol sum over them of
 * sum_j (q_j / d^2)^2 over the ligand atoms within 12 A. */
void orc_desolvation_penalty(const orc_lattice *g, const double *prot_contrib,
                             const uint8_t *prot_shell, int n, const double *x, const double *y,
                             const double *z, const double *q, const double *radius, double r_w,
                             double out[2]) {
  const size_t np = (size_t)g->nx * g->ny * g->nz;
  uint8_t *ls = (uint8_t *)malloc(np);
  orc_masks(g, n, x, y, z, radius, r_w, NULL, ls);
  const double vol = g->step * g->step * g->step;
  double pd = 0.0, ld = 0.0;
  for (int k = 0; k < g->nz; ++k)
    for (int j = 0; j < g->ny; ++j)
      for (int i = 0; i < g->nx; ++i) {
        const size_t idx = i + (size_t)j * g->nx + (size_t)k * g->nx * g->ny;
        if (!(ls[idx] && prot_shell[idx])) continue;
        const double p[3] = {g->o[0] + g->step * i, g->o[1] + g->step * j, g->o[2] + g->step * k};
        for (int a = 0; a < n; ++a) {
          const double dx = p[0] - x[a], dy = p[1] - y[a], dz = p[2] - z[a];
          const double d2 = dx * dx + dy * dy + dz * dz;
          if (d2 < 144.0) {
            const double v = q[a] / d2;
            ld += v * v;
          }
        }
        pd += prot_contrib[idx];
      }
  free(ls);
  out[0] = pd;
  out[1] = orc_desolv_constant() * (vol * ld);
}

/* ---- Monte Carlo chains: replay of a GPU trace ------------------------------
 * One chain of Lds.simulate_lig (src/lds.ml:882-995) frame by frame, in the
 * reference's semantics as the GPU chains implement them: rigid moves on even
 * frames (Move.rand_rot / rand_trans, src/move.ml:14-54, or the Gaussian law),
 * one torsion on odd frames (Mol.tweak_rbond / flip_rbond, src/mol.ml:635-647,
 * the flip cadence of src/lds.ml:783-793); the hard region of interest and the
 * E_inter = 0 resets (reset_run_params, src/lds.ml:652-671, 906-928); the
 * Metropolis test in FP64 (src/lds.ml:931-934); acceptance counted in sliding
 * windows of 100 events (src/SW.ml:7-37) and the step-size adaptation of
 * src/lds.ml:586-621, 962-988.  The random numbers are the GPU's: Philox4x32-10
 * keyed by the seed, counter (chain, frame, draw, 0), two words per uniform
 * with 53 random bits.  The trial poses are rounded to float32 as the GPU
 * stores them.
 *
 * The replay walks the GPU's trace: each frame's proposal is recomputed from
 * the chain's current state and compared bit for bit with the GPU's trial;
 * the trial is scored in FP64 and the outcome (accepted, rejected, reset,
 * chain ended) decided from the FP64 energies.  An outcome whose test lies
 * within e_tol max(|E|, S) of its threshold (Metropolis), or whose trial sits
 * on the cut-off or enclosing-radius boundary, is ambiguous: the replay takes
 * the GPU's outcome there and counts it.  Any other difference is counted as
 * a mismatch, and the replay then follows the GPU so that one difference
 * does not hide the rest. */
static double mc_u01(uint32_t a, uint32_t b) {
  return (double)((((uint64_t)a) << 21) ^ (uint64_t)(b >> 11)) * (1.0 / 9007199254740992.0);
}

static void mc_philox(int b, int step, uint32_t draw, const uint32_t key[2], uint32_t out[4]) {
  const uint32_t c[4] = {(uint32_t)b, (uint32_t)step, draw, 0u};
  orc_philox4x32_10(c, key, out);
}

/* Box-Muller pair from two uniforms */
static void mc_normal2(double u1, double u2, double *n0, double *n1) {
  const double r = sqrt(-2.0 * log(1.0 - u1));
  *n0 = r * cos(2.0 * ORC_PI * u2);
  *n1 = r * sin(2.0 * ORC_PI * u2);
}

static double mc_wrap_pi(double a) {
  a = fmod(a + ORC_PI, 2.0 * ORC_PI);
  if (a < 0.0) a += 2.0 * ORC_PI;
  return a - ORC_PI;
}

/* sliding window: ring of 100 event bits, length, accepts */
typedef struct {
  unsigned char ev[100];
  int head, len, acc;
} mc_window;

static void mc_sw_reset(mc_window *w) { memset(w, 0, sizeof *w); }

static void mc_sw_process(mc_window *w, int evt) {
  if (w->len == 100) w->acc -= w->ev[w->head];
  else w->len += 1;
  w->ev[w->head] = (unsigned char)(evt != 0);
  w->acc += evt != 0;
  w->head = w->head + 1 == 100 ? 0 : w->head + 1;
}

static double mc_sw_ratio(const mc_window *w) { return (double)w->acc / (double)w->len; }

/* the proposal of frame `step` of chain b from its current pose */
static int mc_propose(const orc_mc_params *p, int nrb, int b, int step, int conf_steps,
                      const double *st, const float *cur, float *tr) {
  const int nd = 6 + nrb;
  const uint32_t key[2] = {(uint32_t)(p->seed & 0xffffffffu), (uint32_t)(p->seed >> 32)};
  memcpy(tr, cur, sizeof(float) * nd);
  const int rigid = (step & 1) == 0;
  if (!rigid && nrb == 0) return -2;
  uint32_t r0[4], r1[4];
  mc_philox(b, step, 0u, key, r0);
  mc_philox(b, step, 1u, key, r1);
  if (rigid) {
    double ax, ay, az, th, dt[3];
    if (p->law == 1) {
      double n[6], n6, n7;
      uint32_t r2[4], r3[4];
      mc_normal2(mc_u01(r0[0], r0[1]), mc_u01(r0[2], r0[3]), &n[0], &n[1]);
      mc_normal2(mc_u01(r1[0], r1[1]), mc_u01(r1[2], r1[3]), &n[2], &n[3]);
      mc_philox(b, step, 2u, key, r2);
      mc_normal2(mc_u01(r2[0], r2[1]), mc_u01(r2[2], r2[3]), &n[4], &n[5]);
      double s2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
      const double il = 1.0 / sqrt(s2 > 1e-300 ? s2 : 1e-300);
      ax = n[0] * il;
      ay = n[1] * il;
      az = n[2] * il;
      th = st[0] * n[3];
      dt[0] = st[1] * n[4];
      dt[1] = st[1] * n[5];
      mc_philox(b, step, 3u, key, r3);
      mc_normal2(mc_u01(r3[0], r3[1]), mc_u01(r3[2], r3[3]), &n6, &n7);
      dt[2] = st[1] * n6;
    } else {
      uint32_t r2[4];
      th = (2.0 * mc_u01(r0[0], r0[1]) - 1.0) * st[0];
      int axis = (int)(mc_u01(r0[2], r0[3]) * 3.0);
      if (axis > 2) axis = 2;
      ax = axis == 0;
      ay = axis == 1;
      az = axis == 2;
      dt[0] = (2.0 * mc_u01(r1[0], r1[1]) - 1.0) * st[1];
      dt[1] = (2.0 * mc_u01(r1[2], r1[3]) - 1.0) * st[1];
      mc_philox(b, step, 2u, key, r2);
      dt[2] = (2.0 * mc_u01(r2[0], r2[1]) - 1.0) * st[1];
    }
    /* R' = Rm R (rot.ml:121-146 for Rm, rot.ml:52-66 for R), then
     * Rot.decompose (rot.ml:71-75) */
    double R[9], M[9], Q[9];
    const double u[3] = {ax, ay, az};
    orc_rot_xyz((double)cur[3], (double)cur[4], (double)cur[5], R);
    orc_rot_axis_angle(u, th, M);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        Q[3 * i + j] = M[3 * i] * R[j] + M[3 * i + 1] * R[3 + j] + M[3 * i + 2] * R[6 + j];
    const double beta = atan2(-Q[6], sqrt(Q[0] * Q[0] + Q[3] * Q[3]));
    const double icb = 1.0 / cos(beta);
    tr[3] = (float)atan2(Q[7] * icb, Q[8] * icb);
    tr[4] = (float)beta;
    tr[5] = (float)atan2(Q[3] * icb, Q[0] * icb);
    for (int k = 0; k < 3; ++k) tr[k] = (float)((double)cur[k] + dt[k]);
    return -1;
  }
  int i = (int)(mc_u01(r0[0], r0[1]) * nrb);
  if (i > nrb - 1) i = nrb - 1;
  double d;
  if (p->law == 1) {
    double n0, n1;
    mc_normal2(mc_u01(r0[2], r0[3]), mc_u01(r1[0], r1[1]), &n0, &n1);
    d = st[2 + i] * n0;
  } else {
    const int flip = p->flip_every > 0 && conf_steps > 0 && conf_steps % p->flip_every == 0;
    d = (2.0 * mc_u01(r0[2], r0[3]) - 1.0) * (flip ? ORC_PI : st[2 + i]);
  }
  tr[6 + i] = (float)mc_wrap_pi((double)cur[6 + i] + d);
  return i;
}

/* E, E_inter, the condition scale S, the smallest inter pair r^2 and the
 * enclosing radius of one configuration under the MC pose map */
static void mc_energies(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                        const double *conf, double *E, double *Ei, double *S, double *r2min,
                        double *radius) {
  const int n = lig->m.n;
  const double K = orc_elec_weight();
  double *x = (double *)malloc(sizeof(double) * 3 * n + 1), *y = x + n, *z = x + 2 * n;
  double *t = (double *)malloc(sizeof(double) * 3 * n + 1);
  apply_torsions(lig, conf + 6, t, t + n, t + 2 * n);
  double c[3];
  centroid(n, t, t + n, t + 2 * n, c);
  double rad = 0.0;
  for (int i = 0; i < n; ++i) {
    const double dx = c[0] - t[i], dy = c[1] - t[n + i], dz = c[2] - t[2 * n + i];
    const double d = 0.01 + sqrt(dx * dx + dy * dy + dz * dz);
    if (d > rad) rad = d;
  }
  orc_apply_config(lig, conf, ORC_F_RECENTER, x, y, z);
  double e = 0.0, ei = 0.0, s = 0.0, mn = 1e300, ea;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < prot->n; ++i) {
      const double d[3] = {x[j] - prot->x[i], y[j] - prot->y[i], z[j] - prot->z[i]};
      const double r2 = dot(d, d);
      if (r2 < mn) mn = r2;
      if (ph->inter_form == 0 && !(r2 < 144.0)) continue;
      double x_ij, d_ij, ep;
      orc_pair_params(ph, prot->anum[i], lig->m.anum[j], &x_ij, &d_ij);
      const double qq = K * prot->q[i] * lig->m.q[j];
      pair_energy_grad(ph->dielectric, ph->inter_form == 0, r2, qq, x_ij, d_ij, &ep);
      pair_energy_grad_abs(ph->dielectric, ph->inter_form == 0, r2, qq, x_ij, d_ij, &ea);
      ei += ep;
      s += ea;
    }
  e = ei;
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j) {
      if (!lig->interacting[i * n + j]) continue;
      const double d[3] = {x[i] - x[j], y[i] - y[j], z[i] - z[j]};
      const double r2 = dot(d, d);
      const int shifted = ph->intra_form == 1;
      if (shifted && !(orc_non_zero_dist(sqrt(r2)) < 12.0)) continue;
      double x_ij, d_ij, ep;
      orc_pair_params(ph, lig->m.anum[i], lig->m.anum[j], &x_ij, &d_ij);
      const double qq = K * lig->m.q[i] * lig->m.q[j];
      pair_energy_grad(ph->dielectric, shifted, r2, qq, x_ij, d_ij, &ep);
      pair_energy_grad_abs(ph->dielectric, shifted, r2, qq, x_ij, d_ij, &ea);
      e += ep;
      s += ea;
    }
  *E = e;
  *Ei = ei;
  *S = s;
  *r2min = mn;
  *radius = rad;
  free(t);
  free(x);
}

static int mc_metropolis(double Et, double E0, double u, double kT) {
  return Et <= E0 || u < exp(-(Et - E0) / kT);
}

typedef struct {
  const orc_physics *ph;
  const orc_mol *prot;
  const orc_ligand *lig;
  const orc_mc_params *p;
  int B, steps, b0, b1;
  const float *start, *gpu_trial;
  const double *gpu_E;
  const int *gpu_event;
  float *gen_trial; /* generate mode: the oracle's own trace goes here */
  double *gen_E;
  int *gen_event;
  double e_tol;
  orc_mc_stats st;
} mc_job;

static void *mc_worker(void *arg) {
  mc_job *J = (mc_job *)arg;
  const orc_mc_params *p = J->p;
  const int nrb = J->lig->nrb, nd = 6 + nrb, B = J->B;
  const uint32_t key[2] = {(uint32_t)(p->seed & 0xffffffffu), (uint32_t)(p->seed >> 32)};
  float *cur = (float *)malloc(sizeof(float) * nd), *tr = (float *)malloc(sizeof(float) * nd);
  double *st = (double *)malloc(sizeof(double) * (2 + nrb)), *conf = (double *)malloc(
                                                                   sizeof(double) * nd);
  mc_window *win = (mc_window *)malloc(sizeof(mc_window) * (1 + nrb));
  double *ccur = (double *)malloc(sizeof(double) * nd);
  for (int b = J->b0; b < J->b1; ++b) {
    memcpy(cur, J->start + (size_t)b * nd, sizeof(float) * nd);
    st[0] = p->rot;
    st[1] = p->trans;
    for (int i = 0; i < nrb; ++i) st[2 + i] = p->tors;
    for (int k = 0; k <= nrb; ++k) mc_sw_reset(&win[k]);
    for (int k = 0; k < nd; ++k) ccur[k] = (double)cur[k];
    double E0, Ei0, S0, m0, rad0;
    mc_energies(J->ph, J->prot, J->lig, ccur, &E0, &Ei0, &S0, &m0, &rad0);
    int rigid_steps = 0, conf_steps = 0, stopped = 0;
    for (int step = 0; step < J->steps; ++step) {
      const size_t o = (size_t)step * B + b;
      const int gen = J->gen_trial != NULL;
      const int rigid = (step & 1) == 0;
      int mv = -2;
      if (!stopped) mv = mc_propose(p, nrb, b, step, conf_steps, st, cur, tr);
      else memcpy(tr, cur, sizeof(float) * nd);
      if (gen) memcpy(J->gen_trial + o * nd, tr, sizeof(float) * nd);
      const float *gt = gen ? J->gen_trial + o * nd : J->gpu_trial + o * nd;
      J->st.proposals += 1;
      if (memcmp(tr, gt, sizeof(float) * nd) != 0) {
        J->st.proposal_mismatch += 1;
        memcpy(tr, gt, sizeof(float) * nd);
      }
      int ev = 0, amb = 0;
      double Et = 0, Ei = 0, S = 0, r2m = 0, rad = 0;
      if (stopped) {
        ev = 4;
      } else {
        for (int k = 0; k < nd; ++k) conf[k] = (double)tr[k];
        mc_energies(J->ph, J->prot, J->lig, conf, &Et, &Ei, &S, &r2m, &rad);
        const int too_long = mv >= 0 && rad > 12.0;
        if (mv >= 0 && fabs(rad - 12.0) < 1e-6) amb = 1;
        if (gen) J->gen_E[o] = Et;
        const double gE = gen ? Et : J->gpu_E[o];
        if (isfinite(gE) && isfinite(Et)) {
          const double den = fmax(fabs(Et), S);
          const double err = den > 0 ? fabs(gE - Et) / den : 0.0;
          if (err > J->st.max_rel_err_E) J->st.max_rel_err_E = err;
        }
        int reset = 0;
        if (p->roi_r > 0.0) {
          const double dx = (double)tr[0] - p->roi_c[0], dy = (double)tr[1] - p->roi_c[1],
                       dz = (double)tr[2] - p->roi_c[2];
          const double d = sqrt(dx * dx + dy * dy + dz * dz);
          reset = d > p->roi_r;
          if (fabs(d - p->roi_r) < 1e-9) amb = 1;
        }
        if (!reset && p->reset_zero) {
          if (Ei == 0.0) reset = 1;
          if (fabs(r2m - 144.0) < 1e-3) amb = 1;
        }
        if (reset) {
          ev = 2;
        } else if (too_long && p->too_long_ends) {
          ev = 4;
        } else {
          const int blocked = !isfinite(Et) || too_long;
          int acc = 0;
          if (!blocked) {
            uint32_t r[4];
            mc_philox(b, step, 7u, key, r);
            const double u = mc_u01(r[0], r[1]);
            acc = mc_metropolis(Et, E0, u, p->kT);
            const double dt = J->e_tol * fmax(fabs(Et), S), d0 = J->e_tol * fmax(fabs(E0), S0);
            if (isfinite(E0) &&
                mc_metropolis(Et + dt, E0 - d0, u, p->kT) != mc_metropolis(Et - dt, E0 + d0, u,
                                                                           p->kT))
              amb = 1;
          }
          ev = (acc ? 1 : 0) | (blocked ? 8 : 0);
        }
      }
      if (gen) J->gen_event[o] = ev;
      const int gev = gen ? ev : J->gpu_event[o];
      J->st.decisions += 1;
      if (ev != gev) {
        if (amb) J->st.ambiguous += 1;
        else J->st.decision_mismatch += 1;
        ev = gev; /* follow the GPU */
      } else if (amb) {
        J->st.ambiguous += 1;
      }
      /* apply the outcome */
      if (ev & 4) {
        stopped = 1;
      } else if (ev & 2) {
        J->st.resets += 1;
        memcpy(cur, J->start + (size_t)b * nd, sizeof(float) * 6);
        E0 = INFINITY;
        S0 = 0.0;
        st[0] = p->rot;
        st[1] = p->trans;
        mc_sw_reset(&win[0]);
      } else {
        const int acc = ev & 1;
        if (mv == -1) mc_sw_process(&win[0], acc);
        else if (mv >= 0) mc_sw_process(&win[1 + mv], acc);
        if (acc) {
          memcpy(cur, tr, sizeof(float) * nd);
          E0 = Et;
          S0 = S;
        }
        if (p->adapt && rigid && rigid_steps > 0 && rigid_steps % 100 == 0) {
          const double ratio = mc_sw_ratio(&win[0]);
          if (ratio <= 0.45) {
            st[1] = 0.95 * st[1];
            st[0] = 0.95 * st[0];
            J->st.adapt_events += 1;
          } else if (ratio >= 0.55) {
            st[1] = 1.05 * st[1];
            st[0] = fmin(ORC_PI, 1.05 * st[0]);
            J->st.adapt_events += 1;
          }
        }
        if (p->adapt && acc && mv >= 0 && conf_steps > 0 && conf_steps % (100 * nrb) == 0) {
          for (int i = 0; i < nrb; ++i) {
            const double ratio = mc_sw_ratio(&win[1 + i]);
            if (ratio <= 0.45) st[2 + i] = 0.95 * st[2 + i];
            else if (ratio >= 0.55) st[2 + i] = fmin(ORC_PI, 1.05 * st[2 + i]);
          }
          J->st.adapt_events += 1;
        }
      }
      if (rigid) rigid_steps += 1;
      else conf_steps += 1;
    }
  }
  free(ccur);
  free(win);
  free(conf);
  free(st);
  free(tr);
  free(cur);
  return NULL;
}

static void mc_run_jobs(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                        const orc_mc_params *p, int B, const float *start, int steps,
                        const float *gpu_trial, const double *gpu_E, const int *gpu_event,
                        float *gen_trial, double *gen_E, int *gen_event, double e_tol,
                        int nthreads, orc_mc_stats *out) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > B) nthreads = B > 0 ? B : 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  mc_job *jobs = (mc_job *)calloc(nthreads, sizeof(mc_job));
  for (int t = 0; t < nthreads; ++t) {
    mc_job *j = &jobs[t];
    j->ph = ph;
    j->prot = prot;
    j->lig = lig;
    j->p = p;
    j->B = B;
    j->steps = steps;
    j->b0 = (int)((long)B * t / nthreads);
    j->b1 = (int)((long)B * (t + 1) / nthreads);
    j->start = start;
    j->gpu_trial = gpu_trial;
    j->gpu_E = gpu_E;
    j->gpu_event = gpu_event;
    j->gen_trial = gen_trial;
    j->gen_E = gen_E;
    j->gen_event = gen_event;
    j->e_tol = e_tol;
    if (nthreads == 1) mc_worker(j);
    else pthread_create(&th[t], NULL, mc_worker, j);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  memset(out, 0, sizeof *out);
  for (int t = 0; t < nthreads; ++t) {
    const orc_mc_stats *s = &jobs[t].st;
    out->proposals += s->proposals;
    out->proposal_mismatch += s->proposal_mismatch;
    out->decisions += s->decisions;
    out->decision_mismatch += s->decision_mismatch;
    out->ambiguous += s->ambiguous;
    out->resets += s->resets;
    out->adapt_events += s->adapt_events;
    if (s->max_rel_err_E > out->max_rel_err_E) out->max_rel_err_E = s->max_rel_err_E;
  }
  free(jobs);
  free(th);
}

void orc_mc_replay(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                   const orc_mc_params *p, int B, const float *start, int steps,
                   const float *gpu_trial, const double *gpu_E, const int *gpu_event,
                   double e_tol, int nthreads, orc_mc_stats *out) {
  mc_run_jobs(ph, prot, lig, p, B, start, steps, gpu_trial, gpu_E, gpu_event, NULL, NULL, NULL,
              e_tol, nthreads, out);
}

void orc_mc_run(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                const orc_mc_params *p, int B, const float *start, int steps, float *trial,
                double *E, int *event, int nthreads, orc_mc_stats *out) {
  mc_run_jobs(ph, prot, lig, p, B, start, steps, NULL, NULL, NULL, trial, E, event, 0.0,
              nthreads, out);
}
