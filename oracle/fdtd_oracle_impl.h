/*
 * fdtd_oracle_impl.h -- body of the CPU ORACLE (test infrastructure only).
 *
 * Included by fdtd_oracle_f32.c (REAL=float) and fdtd_oracle_f64.c
 * (REAL=double).  Each function restates one piece of the reference and
 * cites it.  The restatement keeps the reference's structure on purpose:
 * materialised derivative arrays, CPML strips as separate passes, full
 * ParallelStencil `@within` domains (every statement loops over its
 * left-hand-side array), sources added through a spray buffer, records
 * through the transposed interpolation matrix.  It is compiled with
 * -ffp-contract=off so that every expression rounds in the order written.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gpo.h"
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#error "REAL must be defined"
#endif

typedef struct {
  REAL *a;
  int n1, n2, n3;
} arr;

#define AT(f, i, j, k) \
  ((f).a[((size_t)((i)-1)) + (size_t)(f).n1 * (((size_t)((j)-1)) + (size_t)(f).n2 * ((size_t)((k)-1)))])

enum { KF = 0, KV = 1, KH = 2, KI = 3 }; /* n, n+h, n-h, n-2h (src/fields.jl:92-671) */

typedef struct {
  int axis;        /* 0 z, 1 y, 2 x */
  int kz, ky, kx;  /* shape kinds */
  int src;         /* wavefield the derivative is taken of */
  int inner;       /* 1: @d_?i (offset h on the other axes), 0: @d_?a */
} dspec;

/* derivative fields of each physics, in the canonical order of gpo.h
 * (src/fdtd/advance_acou.jl:258-299, src/fdtd/advance_elastic.jl:10-153) */
static const dspec DA2[] = {
    {2, KI, KF, KH, GPO_P, 1},  /* dpdx  = @d_xi(p) */
    {0, KH, KF, KI, GPO_P, 1},  /* dpdz  = @d_zi(p) */
    {2, KF, KF, KF, GPO_VX, 0}, /* dvxdx = @d_xa(vx) */
    {0, KF, KF, KF, GPO_VZ, 0}, /* dvzdz = @d_za(vz) */
};
static const dspec DE2[] = {
    {2, KI, KF, KH, GPO_TAUXX, 1}, /* dtauxxdx = @d_xi(tauxx) */
    {2, KH, KF, KI, GPO_TAUXZ, 0}, /* dtauxzdx = @d_xa(tauxz) */
    {0, KH, KF, KI, GPO_TAUZZ, 1}, /* dtauzzdz = @d_zi(tauzz) */
    {0, KI, KF, KH, GPO_TAUXZ, 0}, /* dtauxzdz = @d_za(tauxz) */
    {2, KF, KF, KF, GPO_VX, 0},    /* dvxdx */
    {0, KF, KF, KF, GPO_VZ, 0},    /* dvzdz */
    {0, KH, KF, KH, GPO_VX, 1},    /* dvxdz = @d_zi(vx) */
    {2, KH, KF, KH, GPO_VZ, 1},    /* dvzdx = @d_xi(vz) */
};
static const dspec DA3[] = {
    {2, KI, KI, KH, GPO_P, 1}, {1, KI, KH, KI, GPO_P, 1}, {0, KH, KI, KI, GPO_P, 1},
    {2, KF, KF, KF, GPO_VX, 0}, {1, KF, KF, KF, GPO_VY, 0}, {0, KF, KF, KF, GPO_VZ, 0},
};
static const dspec DE3[] = {
    {2, KI, KI, KH, GPO_TAUXX, 1}, /* dtauxxdx */
    {2, KI, KH, KI, GPO_TAUXY, 0}, /* dtauxydx */
    {2, KH, KI, KI, GPO_TAUXZ, 0}, /* dtauxzdx */
    {1, KI, KH, KI, GPO_TAUYY, 1}, /* dtauyydy */
    {1, KI, KI, KH, GPO_TAUXY, 0}, /* dtauxydy */
    {1, KH, KI, KI, GPO_TAUYZ, 0}, /* dtauyzdy */
    {0, KH, KI, KI, GPO_TAUZZ, 1}, /* dtauzzdz */
    {0, KI, KH, KI, GPO_TAUYZ, 0}, /* dtauyzdz */
    {0, KI, KI, KH, GPO_TAUXZ, 0}, /* dtauxzdz */
    {2, KF, KF, KF, GPO_VX, 0},    /* dvxdx */
    {1, KF, KF, KF, GPO_VY, 0},    /* dvydy */
    {0, KF, KF, KF, GPO_VZ, 0},    /* dvzdz */
    {1, KI, KH, KH, GPO_VX, 1},    /* dvxdy = @d_yi(vx) */
    {0, KH, KI, KH, GPO_VX, 1},    /* dvxdz = @d_zi(vx) */
    {2, KI, KH, KH, GPO_VY, 1},    /* dvydx = @d_xi(vy) */
    {0, KH, KH, KI, GPO_VY, 1},    /* dvydz = @d_zi(vy) */
    {2, KH, KI, KH, GPO_VZ, 1},    /* dvzdx = @d_xi(vz) */
    {1, KH, KH, KI, GPO_VZ, 1},    /* dvzdy = @d_yi(vz) */
};

/* wavefield shape kinds {z, y, x} (src/fields.jl:92-335) */
static const int FKIND[GPO_NFIELD][3] = {
    {KF, KF, KF}, /* p */
    {KF, KF, KV}, /* vx */
    {KF, KV, KF}, /* vy */
    {KV, KF, KF}, /* vz */
    {KF, KF, KF}, /* tauxx */
    {KF, KF, KF}, /* tauyy */
    {KF, KF, KF}, /* tauzz */
    {KI, KH, KH}, /* tauxy */
    {KH, KI, KH}, /* tauxz */
    {KH, KH, KI}, /* tauyz */
};

typedef struct gpo_ctx {
  gpo_desc d;
  int h, hy;
  REAL dt, dtI, dzI, dyI, dxI;
  int nder;
  const dspec *ds;
  arr mod[3];
  int nmod;
  arr dmod[8];
  int ndmod;
  REAL *pa[18], *pb[18], *pk[18];
  int present[GPO_NFIELD];
  arr w[2][GPO_NFIELD];  /* w1[:t] */
  arr wp[2][GPO_NFIELD]; /* w1[:tp] */
  arr der[2][18];
  arr mem[2][18];
  arr vbuf[3]; /* velocity_buffer of wavefield 1 (gradient scratch) */
  REAL *pv;    /* spray buffer (tauii_buffer / velocity_buffer) */
  unsigned char *pvflag;
  size_t pvlen;
  int nshots;
  REAL **bstore; /* boundary store per shot */
  REAL **hist;   /* forward history per shot (GPO_FORWARD_HIST) */
  int snap_field, nsnap, snap_its[64]; /* snaps_save! (fdtd.jl:586-591) */
  REAL **snaps;  /* per shot: nsnap copies of wavefield 1's snap_field */
  int illum_on;   /* illum_flag: compute_illum! (fdtd.jl:571-582) */
  double **illum; /* per shot: sum over the steps of p^2 of wavefield 1 */
  size_t hstep;  /* REALs per step in the history: p, vx, [vy,] vz */
  size_t bstep;  /* REALs per time step in the store */
  size_t bsnap;  /* REALs of the final snapshots */
  int imaging;   /* 0 the reference's imaging condition, 1 the
                    FD-consistent rho term (gpo_set_imaging) */
  arr born[4];   /* GPO_BORN secondary-source ratios: p, vx, vy, vz */
  int have_born;
  REAL *srcamt;  /* elastic history adjoint: stress-source amounts of the
                    forward step being reversed, per normal-stress cell */
} ctx;

static int nk(const ctx *c, int kind, int n, int dimactive) {
  if (!dimactive) return 1;
  switch (kind) {
    case KV: return n + c->h;
    case KH: return n - c->h;
    case KI: return n - 2 * c->h;
    default: return n;
  }
}

static arr mkarr(const ctx *c, int kz, int ky, int kx) {
  arr r;
  r.n1 = nk(c, kz, c->d.nz, 1);
  r.n2 = nk(c, ky, c->d.ny, c->d.ndim == 3);
  r.n3 = nk(c, kx, c->d.nx, 1);
  r.a = (REAL *)calloc((size_t)r.n1 * r.n2 * r.n3, sizeof(REAL));
  return r;
}
static size_t alen(arr a) { return (size_t)a.n1 * a.n2 * a.n3; }
static void azero(arr a) {
  if (a.a) memset(a.a, 0, alen(a) * sizeof(REAL));
}
static void acopy(arr dst, arr src) { memcpy(dst.a, src.a, alen(src) * sizeof(REAL)); }

/* staggered difference, src/fdtd/diff2D.jl:30-207 (same in diff3D.jl) */
static inline REAL stencil(int order, const REAL *a, ptrdiff_t s) {
  switch (order) {
    case 2: return a[s] - a[0];
    case 4: return a[2 * s] * (REAL)27 - a[s] * (REAL)27 + a[0] - a[3 * s];
    case 6:
      return a[3 * s] * (REAL)2250 - a[2 * s] * (REAL)2250 + a[s] * (REAL)125 - a[4 * s] * (REAL)125 +
             a[5 * s] * (REAL)9 - a[0] * (REAL)9;
    default:
      return a[4 * s] * (REAL)128625 - a[3 * s] * (REAL)128625 + a[2 * s] * (REAL)8575 -
             a[5 * s] * (REAL)8575 + a[6 * s] * (REAL)1029 - a[s] * (REAL)1029 + a[0] * (REAL)75 -
             a[7 * s] * (REAL)75;
  }
}

/* @all(out) = @d_{axis}{a|i}(in) * dsI */
static void deriv(const ctx *c, arr out, arr in, const dspec *s, REAL dsI) {
  const int h = c->h, order = c->d.order;
  const int oz = (s->inner && s->axis != 0) ? h : 0;
  const int oy = (s->inner && s->axis != 1 && c->d.ndim == 3) ? h : 0;
  const int ox = (s->inner && s->axis != 2) ? h : 0;
  const ptrdiff_t st = s->axis == 0 ? 1 : s->axis == 1 ? (ptrdiff_t)in.n1 : (ptrdiff_t)in.n1 * in.n2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ix = 1; ix <= out.n3; ix++)
    for (int iy = 1; iy <= out.n2; iy++)
      for (int iz = 1; iz <= out.n1; iz++) {
        const REAL *a = &AT(in, iz + oz, iy + oy, ix + ox);
        AT(out, iz, iy, ix) = stencil(order, a, st) * dsI;
      }
}

static int axis_face(int axis, int ismax) {
  static const int f[3][2] = {{GPO_ZMIN, GPO_ZMAX}, {GPO_YMIN, GPO_YMAX}, {GPO_XMIN, GPO_XMAX}};
  return f[axis][ismax];
}

/* memory{x,y,z}! (src/fdtd/cpml.jl:158-215): on the first and the last npml
 * entries of the derivative axis, psi = b psi + a d; d = d kI + psi. */
static void memory(const ctx *c, arr psi, arr d, int axis, const REAL *a, const REAL *b, const REAL *kI) {
  const int npml = c->d.npml;
  for (int side = 0; side < 2; side++) {
    if (!(c->d.pml_faces & axis_face(axis, side))) continue;
    const int moff = side ? npml : 0;
    const int nd = axis == 0 ? d.n1 : axis == 1 ? d.n2 : d.n3;
    const int doff = side ? nd - npml : 0;
    const int r1 = axis == 0 ? npml : psi.n1, r2 = axis == 1 ? npml : psi.n2, r3 = axis == 2 ? npml : psi.n3;
#pragma omp parallel for collapse(2) schedule(static)
    for (int ix = 1; ix <= r3; ix++)
      for (int iy = 1; iy <= r2; iy++)
        for (int iz = 1; iz <= r1; iz++) {
          const int i = axis == 0 ? iz : axis == 1 ? iy : ix;
          REAL *m = &AT(psi, axis == 0 ? iz + moff : iz, axis == 1 ? iy + moff : iy, axis == 2 ? ix + moff : ix);
          REAL *dd = &AT(d, axis == 0 ? doff + iz : iz, axis == 1 ? doff + iy : iy, axis == 2 ? doff + ix : ix);
          const int j = i + moff - 1;
          *m = b[j] * *m + a[j] * *dd;
          *dd = *dd * kI[j] + *m;
        }
  }
}

/* dirichlet{z,y,x}{min,max}! (src/fdtd/dirichlet.jl:1-79) applied in the
 * order of update_v! (src/fdtd/advance_acou.jl:50-57, :155-192). */
static void dirichlet(const ctx *c, arr *w) {
  const int order = c->d.order, fdh = order / 2;
  const int three = c->d.ndim == 3;
  const int n[3] = {c->d.nz, c->d.ny, c->d.nx};
  const int vid[3] = {GPO_VZ, GPO_VY, GPO_VX};
  const int seq[6][2] = {{2, 0}, {2, 1}, {1, 0}, {1, 1}, {0, 0}, {0, 1}}; /* x, y, z; min, max */
  for (int q = 0; q < 6; q++) {
    const int axis = seq[q][0], ismax = seq[q][1];
    if (axis == 1 && !three) continue;
    if (!(c->d.rigid_faces & axis_face(axis, ismax))) continue;
    /* the two "other" axes: launch ranges 1:n of those axes */
    const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
    const int na = (oa == 1 && !three) ? 1 : n[oa], nb = n[ob];
    arr v = w[vid[axis]];
    const int nn = n[axis];
#pragma omp parallel for collapse(2) schedule(static)
    for (int jb = 1; jb <= nb; jb++)
      for (int ja = 1; ja <= na; ja++) {
        int idx[3];
        idx[oa] = ja;
        idx[ob] = jb;
        /* other velocity components set to zero at 1 (min) or n (max) */
        for (int o = 0; o < 3; o++) {
          if (o == axis || (o == 1 && !three)) continue;
          arr u = w[vid[o]];
          idx[axis] = ismax ? nn : 1;
          AT(u, idx[0], three ? idx[1] : 1, idx[2]) = (REAL)0;
        }
        for (int ifd = 1; ifd <= fdh; ifd++) {
          int g, s;
          if (!ismax) {
            g = ifd;
            s = order + 1 - ifd;
          } else {
            g = nn + order - ifd;
            s = nn + ifd - 1;
          }
          int ig[3] = {idx[0], idx[1], idx[2]}, is[3] = {idx[0], idx[1], idx[2]};
          ig[axis] = g;
          is[axis] = s;
          AT(v, ig[0], three ? ig[1] : 1, ig[2]) = -AT(v, is[0], three ? is[1] : 1, is[2]);
        }
      }
  }
}

/* ------------------------------------------------------------------ */
/* medium: update_dmod! (src/fdtd/medium.jl:143-221)                   */
/* ------------------------------------------------------------------ */
static void store_invav(const ctx *c, arr out, arr rho, int axis) {
  /* out = dt / @av_{x,y,z}i(rho)  (diff2D.jl:226-233, diff3D.jl:324-335) */
  const int h = c->h, three = c->d.ndim == 3;
  const REAL dt = c->dt;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ix = 1; ix <= out.n3; ix++)
    for (int iy = 1; iy <= out.n2; iy++)
      for (int iz = 1; iz <= out.n1; iz++) {
        int z = iz + (axis != 0 ? h : 0), y = three ? iy + (axis != 1 ? h : 0) : 1, x = ix + (axis != 2 ? h : 0);
        REAL a0 = AT(rho, z, y, x);
        REAL a1 = AT(rho, z + (axis == 0), y + (axis == 1), x + (axis == 2));
        AT(out, iz, iy, ix) = dt / ((a0 + a1) * (REAL)0.5);
      }
}

static void store_invav4(const ctx *c, arr out, arr b, int which) {
  /* which: 0 @av (2-D), 1 @av_xzi, 2 @av_xyi, 3 @av_yzi (diff3D.jl:336-377) */
  const int h = c->h;
  const REAL dt = c->dt;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ix = 1; ix <= out.n3; ix++)
    for (int iy = 1; iy <= out.n2; iy++)
      for (int iz = 1; iz <= out.n1; iz++) {
        REAL s;
        if (which == 0) {
          s = (AT(b, iz, 1, ix) + AT(b, iz + 1, 1, ix) + AT(b, iz, 1, ix + 1) + AT(b, iz + 1, 1, ix + 1)) * (REAL)0.25;
        } else if (which == 1) {
          int y = iy + h;
          s = (AT(b, iz, y, ix) + AT(b, iz + 1, y, ix) + AT(b, iz, y, ix + 1) + AT(b, iz + 1, y, ix + 1)) * (REAL)0.25;
        } else if (which == 2) {
          int z = iz + h;
          s = (AT(b, z, iy, ix) + AT(b, z, iy + 1, ix) + AT(b, z, iy, ix + 1) + AT(b, z, iy + 1, ix + 1)) * (REAL)0.25;
        } else {
          int x = ix + h;
          s = (AT(b, iz, iy, x) + AT(b, iz + 1, iy, x) + AT(b, iz, iy + 1, x) + AT(b, iz + 1, iy + 1, x)) * (REAL)0.25;
        }
        AT(out, iz, iy, ix) = dt / s;
      }
}

static void update_dmod(ctx *c) {
  const int three = c->d.ndim == 3;
  const REAL dt = c->dt;
  if (c->d.physics == GPO_ACOUSTIC) {
    /* [:dtinvavxirho, (:dtinvavyirho), :dtinvavzirho, :dtK] on [dpdx, (dpdy), dpdz, p] */
    int k = 0;
    c->dmod[k] = mkarr(c, c->ds[0].kz, c->ds[0].ky, c->ds[0].kx);
    store_invav(c, c->dmod[k++], c->mod[1], 2);
    if (three) {
      c->dmod[k] = mkarr(c, c->ds[1].kz, c->ds[1].ky, c->ds[1].kx);
      store_invav(c, c->dmod[k++], c->mod[1], 1);
    }
    const dspec *dz = &c->ds[three ? 2 : 1];
    c->dmod[k] = mkarr(c, dz->kz, dz->ky, dz->kx);
    store_invav(c, c->dmod[k++], c->mod[1], 0);
    c->dmod[k] = mkarr(c, KF, KF, KF);
    arr K = c->dmod[k++];
    for (size_t i = 0; i < alen(K); i++) {
      REAL t = (REAL)1 / c->mod[0].a[i]; /* broadcast!(inv, dtK, invK) */
      K.a[i] = t * dt;                   /* rmul!(dtK, dt) */
    }
    c->ndmod = k;
  } else {
    /* 2-D: [:dtinvavxirho, :dtinvavzirho, :dtavmu, :dtM, :dtlambda]
     * 3-D: [:dtinvavxirho, :dtinvavyirho, :dtinvavzirho, :dtavxzimu,
     *       :dtavxyimu, :dtavyzimu, :dtM, :dtlambda]                 */
    int k = 0;
    c->dmod[k] = mkarr(c, c->ds[0].kz, c->ds[0].ky, c->ds[0].kx); /* dtauxxdx grid */
    store_invav(c, c->dmod[k++], c->mod[2], 2);
    if (three) {
      c->dmod[k] = mkarr(c, c->ds[3].kz, c->ds[3].ky, c->ds[3].kx); /* dtauyydy grid */
      store_invav(c, c->dmod[k++], c->mod[2], 1);
      c->dmod[k] = mkarr(c, c->ds[6].kz, c->ds[6].ky, c->ds[6].kx); /* dtauzzdz grid */
      store_invav(c, c->dmod[k++], c->mod[2], 0);
      c->dmod[k] = mkarr(c, KH, KI, KH); /* dvxdz grid */
      store_invav4(c, c->dmod[k++], c->mod[1], 1);
      c->dmod[k] = mkarr(c, KI, KH, KH); /* dvxdy grid */
      store_invav4(c, c->dmod[k++], c->mod[1], 2);
      c->dmod[k] = mkarr(c, KH, KH, KI); /* dvydz grid */
      store_invav4(c, c->dmod[k++], c->mod[1], 3);
    } else {
      c->dmod[k] = mkarr(c, c->ds[2].kz, c->ds[2].ky, c->ds[2].kx); /* dtauzzdz grid */
      store_invav(c, c->dmod[k++], c->mod[2], 0);
      c->dmod[k] = mkarr(c, KH, KF, KH); /* dvxdz grid */
      store_invav4(c, c->dmod[k++], c->mod[1], 0);
    }
    arr M = mkarr(c, KF, KF, KF), L = mkarr(c, KF, KF, KF);
    for (size_t i = 0; i < alen(M); i++) {
      REAL il = c->mod[0].a[i], im = c->mod[1].a[i];
      L.a[i] = ((REAL)1 / il) * dt;
      /* inv(invλ) + 2.0*inv(invμ) is evaluated in Float64 (Float64 literal) */
      double m64 = (double)((REAL)1 / il) + 2.0 * (double)((REAL)1 / im);
      M.a[i] = (REAL)m64 * dt;
    }
    c->dmod[k++] = M;
    c->dmod[k++] = L;
    c->ndmod = k;
  }
}

/* ------------------------------------------------------------------ */
/* sources and receivers                                               */
/* ------------------------------------------------------------------ */

/* pv = S * w[it]  (mul!(pv_vec, ssprayw, w), src/fdtd/source.jl:71,136) and
 * the muladd_* kernels (src/fdtd/source.jl:160-177) restricted to the cells
 * the spray touches (pv is zero elsewhere, so the result is identical). */
static int is_velocity(int f) { return f == GPO_VX || f == GPO_VY || f == GPO_VZ; }
static int is_stress_src(int f) { return f == GPO_P || f == GPO_TAUXX || f == GPO_TAUYY || f == GPO_TAUZZ; }

static void spray(ctx *c, const gpo_proj *s, int it) {
  const REAL *w = (const REAL *)s->data + (size_t)it; /* column j at w[j*nt] */
  const REAL *v = (const REAL *)s->nzval;
  for (int j = 0; j < s->n; j++) {
    REAL wj = w[(size_t)j * c->d.nt];
    for (int64_t k = s->colptr[j]; k < s->colptr[j + 1]; k++) c->pv[s->rowval[k]] += v[k] * wj;
  }
}
static void spray_clear(ctx *c, const gpo_proj *s) {
  for (int j = 0; j < s->n; j++)
    for (int64_t k = s->colptr[j]; k < s->colptr[j + 1]; k++) {
      c->pv[s->rowval[k]] = 0;
      c->pvflag[s->rowval[k]] = 0;
    }
}

static void add_stress_source(ctx *c, arr *w, const gpo_proj *s, int it) {
  spray(c, s, it);
  const int three = c->d.ndim == 3;
  arr dK = c->dmod[c->ndmod - (c->d.physics == GPO_ACOUSTIC ? 1 : 2)]; /* dtK or dtM */
  int targets[3], nt_ = 0;
  if (c->d.physics == GPO_ACOUSTIC)
    targets[nt_++] = GPO_P;
  else {
    targets[nt_++] = GPO_TAUXX;
    if (three) targets[nt_++] = GPO_TAUYY;
    targets[nt_++] = GPO_TAUZZ;
  }
  for (int q = 0; q < nt_; q++) {
    arr f = w[targets[q]];
    for (int j = 0; j < s->n; j++)
      for (int64_t k = s->colptr[j]; k < s->colptr[j + 1]; k++) {
        int64_t r = s->rowval[k];
        if (c->pvflag[r] == q + 1) continue;
        c->pvflag[r] = (unsigned char)(q + 1);
        f.a[r] = f.a[r] + (c->pv[r] * dK.a[r]); /* @all(pw) + (@all(pv) * @all(dtK)) */
      }
  }
  spray_clear(c, s);
}

static void add_velocity_source(ctx *c, arr *w, const gpo_proj *s, int it) {
  spray(c, s, it);
  const int h = c->h, three = c->d.ndim == 3;
  arr v = w[s->field], rho = c->mod[c->d.physics == GPO_ACOUSTIC ? 1 : 2];
  const int axis = s->field == GPO_VZ ? 0 : s->field == GPO_VY ? 1 : 2;
  for (int j = 0; j < s->n; j++)
    for (int64_t k = s->colptr[j]; k < s->colptr[j + 1]; k++) {
      int64_t r = s->rowval[k];
      if (c->pvflag[r]) continue;
      c->pvflag[r] = 1;
      /* 1-based (i1, i2, i3) of r in v */
      int i1 = (int)(r % v.n1) + 1;
      int i2 = (int)((r / v.n1) % v.n2) + 1;
      int i3 = (int)(r / ((int64_t)v.n1 * v.n2)) + 1;
      /* @inn domain: i = i0 + h with i0 <= n - 2h on every active axis */
      if (i1 - h < 1 || i1 - h > v.n1 - 2 * h) continue;
      if (three && (i2 - h < 1 || i2 - h > v.n2 - 2 * h)) continue;
      if (i3 - h < 1 || i3 - h > v.n3 - 2 * h) continue;
      /* @av_{x,y,z}i(rho) at the @inn cell: (iz, iy, ix) = i - h */
      int z = i1 - h, y = three ? i2 - h : 1, x = i3 - h;
      int zz = z + (axis != 0 ? h : 0), yy = three ? y + (axis != 1 ? h : 0) : 1, xx = x + (axis != 2 ? h : 0);
      REAL a0 = AT(rho, zz, yy, xx);
      REAL a1 = AT(rho, zz + (axis == 0), yy + (axis == 1), xx + (axis == 2));
      REAL av = (a0 + a1) * (REAL)0.5;
      v.a[r] = v.a[r] + (c->pv[r] / av * c->dt);
    }
  spray_clear(c, s);
}

/* record! (src/fdtd/receiver.jl:3-15): rec[it] = transpose(W) * vec(field) */
static void record(const ctx *c, arr *w, gpo_proj *r, int it) {
  const REAL *v = (const REAL *)r->nzval;
  REAL *out = (REAL *)r->data;
  arr f = w[r->field];
  for (int j = 0; j < r->n; j++) {
    REAL s = 0;
    for (int64_t k = r->colptr[j]; k < r->colptr[j + 1]; k++) s += v[k] * f.a[r->rowval[k]];
    out[(size_t)j * c->d.nt + it] = s;
  }
}

/* ------------------------------------------------------------------ */
/* the four sub-steps of one wavefield                                 */
/* ------------------------------------------------------------------ */

static REAL dsI_of(const ctx *c, int axis) { return axis == 0 ? c->dzI : axis == 1 ? c->dyI : c->dxI; }

/* update_dstress! : derivatives of the stress (or p) plus CPML */
static void update_dstress(ctx *c, int ipw) {
  const int nstress = c->d.physics == GPO_ACOUSTIC ? c->d.ndim : (c->d.ndim == 2 ? 4 : 9);
  for (int q = 0; q < nstress; q++) {
    const dspec *s = &c->ds[q];
    deriv(c, c->der[ipw][q], c->w[ipw][s->src], s, dsI_of(c, s->axis));
  }
  for (int q = 0; q < nstress; q++)
    memory(c, c->mem[ipw][q], c->der[ipw][q], c->ds[q].axis, c->pa[q], c->pb[q], c->pk[q]);
}

/* update_dv! : derivatives of the velocities plus CPML */
static void update_dv(ctx *c, int ipw) {
  const int nstress = c->d.physics == GPO_ACOUSTIC ? c->d.ndim : (c->d.ndim == 2 ? 4 : 9);
  for (int q = nstress; q < c->nder; q++) {
    const dspec *s = &c->ds[q];
    deriv(c, c->der[ipw][q], c->w[ipw][s->src], s, dsI_of(c, s->axis));
  }
  for (int q = nstress; q < c->nder; q++)
    memory(c, c->mem[ipw][q], c->der[ipw][q], c->ds[q].axis, c->pa[q], c->pb[q], c->pk[q]);
}

/* update_v! : compute_v! then the rigid (Dirichlet) faces */
static void update_v(ctx *c, int ipw) {
  const int h = c->h, hy = c->hy, three = c->d.ndim == 3;
  arr *w = c->w[ipw], *D = c->der[ipw];
  const int vids[3] = {GPO_VX, GPO_VY, GPO_VZ};
  for (int q = 0; q < 3; q++) {
    if (q == 1 && !three) continue;
    arr v = w[vids[q]];
    /* coefficient index in dmod: x -> 0, y -> 1, z -> 1 (2-D) or 2 (3-D) */
    arr cf = c->dmod[q == 0 ? 0 : q == 1 ? 1 : (three ? 2 : 1)];
    const int r1 = v.n1 - 2 * h, r2 = three ? v.n2 - 2 * hy : 1, r3 = v.n3 - 2 * h;
#pragma omp parallel for collapse(2) schedule(static)
    for (int ix = 1; ix <= r3; ix++)
      for (int iy = 1; iy <= r2; iy++)
        for (int iz = 1; iz <= r1; iz++) {
          REAL *vv = &AT(v, iz + h, iy + hy, ix + h);
          REAL cc = AT(cf, iz, iy, ix);
          if (c->d.physics == GPO_ACOUSTIC) {
            /* @inn(v) = @inn(v) + @all(c) * @all(dp) (advance_acou.jl:273-284) */
            int di = three ? q : (q == 0 ? 0 : 1);
            *vv = *vv + cc * AT(D[di], iz, iy, ix);
          } else if (!three) {
            /* advance_elastic.jl:96-110 */
            if (q == 0)
              *vv = *vv - cc * (AT(D[0], iz, iy, ix) + AT(D[3], iz, iy, ix));
            else
              *vv = *vv - cc * (AT(D[1], iz, iy, ix) + AT(D[2], iz, iy, ix));
          } else {
            /* advance_elastic.jl:69-94 */
            if (q == 0)
              *vv = *vv - cc * (AT(D[0], iz, iy, ix) + AT(D[4], iz, iy, ix) + AT(D[8], iz, iy, ix));
            else if (q == 1)
              *vv = *vv - cc * (AT(D[1], iz, iy, ix) + AT(D[3], iz, iy, ix) + AT(D[7], iz, iy, ix));
            else
              *vv = *vv - cc * (AT(D[2], iz, iy, ix) + AT(D[5], iz, iy, ix) + AT(D[6], iz, iy, ix));
          }
        }
  }
  dirichlet(c, w);
}

/* update_stress! : compute_p! / compute_stressii! + compute_stressij! +
 * free surface (advance_acou.jl:303-313, advance_elastic.jl:155-230) */
static void update_stress(ctx *c, int ipw) {
  const int three = c->d.ndim == 3;
  arr *w = c->w[ipw], *D = c->der[ipw];
  if (c->d.physics == GPO_ACOUSTIC) {
    arr p = w[GPO_P], K = c->dmod[c->ndmod - 1];
    const int o = three ? 3 : 2; /* first velocity derivative */
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < alen(p); i++) {
      if (three) /* (dvxdx + dvzdz + dvydy) */
        p.a[i] = p.a[i] + (D[o].a[i] + D[o + 2].a[i] + D[o + 1].a[i]) * K.a[i];
      else
        p.a[i] = p.a[i] + (D[o].a[i] + D[o + 1].a[i]) * K.a[i];
    }
    return;
  }
  arr M = c->dmod[c->ndmod - 2], L = c->dmod[c->ndmod - 1];
  if (!three) {
    arr txx = w[GPO_TAUXX], tzz = w[GPO_TAUZZ], txz = w[GPO_TAUXZ];
    arr dvxdx = D[4], dvzdz = D[5], dvxdz = D[6], dvzdx = D[7], mu = c->dmod[2];
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < alen(txx); i++) {
      txx.a[i] = txx.a[i] - (M.a[i] * dvxdx.a[i]) - (L.a[i] * (dvzdz.a[i]));
      tzz.a[i] = tzz.a[i] - (M.a[i] * dvzdz.a[i]) - (L.a[i] * (dvxdx.a[i]));
    }
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < alen(txz); i++) txz.a[i] = txz.a[i] - mu.a[i] * (dvxdz.a[i] + dvzdx.a[i]);
    if (c->d.free_faces & GPO_ZMIN) {
      for (int ix = 1; ix <= tzz.n3; ix++) AT(tzz, 1, 1, ix) = -AT(tzz, 2, 1, ix);
      for (int ix = 1; ix <= txz.n3; ix++) AT(txz, 1, 1, ix) = (REAL)0;
    }
    return;
  }
  arr txx = w[GPO_TAUXX], tyy = w[GPO_TAUYY], tzz = w[GPO_TAUZZ];
  arr txy = w[GPO_TAUXY], txz = w[GPO_TAUXZ], tyz = w[GPO_TAUYZ];
  arr dvxdx = D[9], dvydy = D[10], dvzdz = D[11];
  arr dvxdy = D[12], dvxdz = D[13], dvydx = D[14], dvydz = D[15], dvzdx = D[16], dvzdy = D[17];
  arr mxz = c->dmod[3], mxy = c->dmod[4], myz = c->dmod[5];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < alen(txx); i++) {
    txx.a[i] = txx.a[i] - (M.a[i] * dvxdx.a[i]) - (L.a[i] * (dvydy.a[i] + dvzdz.a[i]));
    tyy.a[i] = tyy.a[i] - (M.a[i] * dvydy.a[i]) - (L.a[i] * (dvxdx.a[i] + dvzdz.a[i]));
    tzz.a[i] = tzz.a[i] - (M.a[i] * dvzdz.a[i]) - (L.a[i] * (dvydy.a[i] + dvxdx.a[i]));
  }
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < alen(txz); i++) txz.a[i] = txz.a[i] - mxz.a[i] * (dvxdz.a[i] + dvzdx.a[i]);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < alen(txy); i++) txy.a[i] = txy.a[i] - mxy.a[i] * (dvxdy.a[i] + dvydx.a[i]);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < alen(tyz); i++) tyz.a[i] = tyz.a[i] - myz.a[i] * (dvydz.a[i] + dvzdy.a[i]);
  if (c->d.free_faces & GPO_ZMIN) {
    for (int ix = 1; ix <= tzz.n3; ix++)
      for (int iy = 1; iy <= tzz.n2; iy++) AT(tzz, 1, iy, ix) = -AT(tzz, 2, iy, ix);
    for (int ix = 1; ix <= txz.n3; ix++)
      for (int iy = 1; iy <= txz.n2; iy++) AT(txz, 1, iy, ix) = (REAL)0;
    for (int ix = 1; ix <= tyz.n3; ix++)
      for (int iy = 1; iy <= tyz.n2; iy++) AT(tyz, 1, iy, ix) = (REAL)0;
  }
}

/* ------------------------------------------------------------------ */
/* boundary store for time reversal (src/fdtd/boundary.jl)             */
/* ------------------------------------------------------------------ */
static int nsaved(const ctx *c, int *ids) {
  if (c->d.physics == GPO_ACOUSTIC) {
    ids[0] = GPO_P;
    return 1;
  }
  ids[0] = GPO_TAUXX;
  ids[1] = GPO_TAUXZ;
  ids[2] = GPO_TAUZZ;
  return 3;
}
static size_t strip_len(const ctx *c, arr f, int axis) {
  size_t n = 2 * (size_t)c->d.nbound;
  if (axis != 0) n *= f.n1;
  if (axis != 1) n *= f.n2;
  if (axis != 2) n *= f.n3;
  return n;
}
/* save (dir=0): b = d strips; force (dir=1): d = b  (boundary.jl:17-52).
 * np = npml if the MIN face of that axis is a PML face (both ends). */
static REAL *strip_copy(const ctx *c, arr f, int axis, REAL *b, int dir) {
  const int nb = c->d.nbound;
  const int np = (c->d.pml_faces & axis_face(axis, 0)) ? c->d.npml : 0;
  const int nf = axis == 0 ? f.n1 : axis == 1 ? f.n2 : f.n3;
  arr B;
  B.a = b;
  B.n1 = axis == 0 ? 2 * nb : f.n1;
  B.n2 = axis == 1 ? 2 * nb : f.n2;
  B.n3 = axis == 2 ? 2 * nb : f.n3;
  for (int side = 0; side < 2; side++) {
    const int boff = side ? nb : 0, doff = side ? nf - np - nb : np;
    const int r1 = axis == 0 ? nb : f.n1, r2 = axis == 1 ? nb : f.n2, r3 = axis == 2 ? nb : f.n3;
    for (int ix = 1; ix <= r3; ix++)
      for (int iy = 1; iy <= r2; iy++)
        for (int iz = 1; iz <= r1; iz++) {
          REAL *bb = &AT(B, iz + (axis == 0) * boff, iy + (axis == 1) * boff, ix + (axis == 2) * boff);
          REAL *dd = &AT(f, iz + (axis == 0) * doff, iy + (axis == 1) * doff, ix + (axis == 2) * doff);
          if (dir == 0)
            *bb = *dd;
          else
            *dd = *bb;
        }
  }
  return b + alen(B);
}
static void boundary_save(ctx *c, int ishot, int it) {
  /* boundary_save! (boundary.jl:217-264): strips then rmul!(-1) */
  int ids[3];
  const int n = nsaved(c, ids);
  REAL *b = c->bstore[ishot] + (size_t)(it - 1) * c->bstep;
  for (int q = 0; q < n; q++) {
    arr f = c->w[0][ids[q]];
    for (int axis = 2; axis >= 0; axis--) {
      if (axis == 1 && c->d.ndim == 2) continue;
      REAL *b0 = b;
      b = strip_copy(c, f, axis, b, 0);
      for (REAL *t = b0; t < b; t++) *t = -*t;
    }
  }
}
static void boundary_force(ctx *c, int ishot, int it) {
  /* boundary_force! (boundary.jl:115-169): x strips, (y), then z strips */
  int ids[3];
  const int n = nsaved(c, ids);
  REAL *b = c->bstore[ishot] + (size_t)(it - 1) * c->bstep;
  for (int q = 0; q < n; q++) {
    arr f = c->w[0][ids[q]];
    for (int axis = 2; axis >= 0; axis--) {
      if (axis == 1 && c->d.ndim == 2) continue;
      b = strip_copy(c, f, axis, b, 1);
    }
  }
}
static REAL *snap_base(ctx *c, int ishot) { return c->bstore[ishot] + (size_t)c->d.nt * c->bstep; }
static void snap_io(ctx *c, int ishot, int tau, int dir) {
  /* boundary_save_snap_{tau,v}! / boundary_force_snap_{tau,v}! (boundary.jl:172-306) */
  int ids[3];
  const int ns = nsaved(c, ids);
  REAL *b = snap_base(c, ishot);
  const int vids[3] = {GPO_VX, GPO_VY, GPO_VZ};
  for (int q = 0; q < ns; q++) {
    arr f = c->w[0][ids[q]];
    if (tau) {
      if (dir == 0)
        for (size_t i = 0; i < alen(f); i++) b[i] = -f.a[i];
      else
        memcpy(f.a, b, alen(f) * sizeof(REAL));
    }
    b += alen(f);
  }
  for (int q = 0; q < 3; q++) {
    if (q == 1 && c->d.ndim == 2) continue;
    arr f = c->w[0][vids[q]];
    if (!tau) {
      if (dir == 0)
        memcpy(b, f.a, alen(f) * sizeof(REAL));
      else
        memcpy(f.a, b, alen(f) * sizeof(REAL));
    }
    b += alen(f);
  }
}

/* ------------------------------------------------------------------ */
/* gradient (src/fdtd/gradient.jl:17-64), acoustic 2-D                 */
/* ------------------------------------------------------------------ */
static void compute_gradient_elastic(ctx *c, REAL *gL, REAL *gM, REAL *gR, const REAL *A);

static void rho_gather(ctx *c, REAL *gR) {
  const int three = c->d.ndim == 3;
  /* FD-consistent rho term (no reference counterpart): rho at cell
   * (R, [Y,] C) enters the update coefficient dt / avg(rho) of the
   * velocity cells two and three cells further along each axis (vx
   * (R, C+2), (R, C+3); vz (R+2, C), (R+3, C); vy (Y+2), (Y+3):
   * store_invav averages rho at i-3 and i-2 for velocity cell i), each
   * with weight 1/2 and only where that velocity cell is updated (the
   * @inn domain of update_v!: rows 4..nz-3 for vx and vy, 4..nz for vz,
   * and so on along each axis). */
  arr bx = c->vbuf[0], bz = c->vbuf[1], by = c->vbuf[2];
  const int nz = c->d.nz, nx = c->d.nx, ny = three ? c->d.ny : 1;
  /* update domains: [lo, hi] per axis (z, y, x) of vx, vy, vz */
  const int hz = nz - 3, hyy = ny - 3, hx = nx - 3;
#define IN(a, lo, hi) ((a) >= (lo) && (a) <= (hi))
  for (int C = 1; C <= nx; C++)
    for (int Y = 1; Y <= ny; Y++)
      for (int R = 1; R <= nz; R++) {
        const int yin = !three || IN(Y, 4, hyy);
        REAL avx = 0, avz = 0, avy = 0;
        if (IN(R, 4, hz) && yin) {
          REAL b2 = IN(C + 2, 4, nx) ? AT(bx, R, Y, C + 2) : (REAL)0;
          REAL b3 = IN(C + 3, 4, nx) ? AT(bx, R, Y, C + 3) : (REAL)0;
          avx = (b2 + b3) * (REAL)0.5;
        }
        if (IN(C, 4, hx) && yin) {
          REAL b2 = IN(R + 2, 4, nz) ? AT(bz, R + 2, Y, C) : (REAL)0;
          REAL b3 = IN(R + 3, 4, nz) ? AT(bz, R + 3, Y, C) : (REAL)0;
          avz = (b2 + b3) * (REAL)0.5;
        }
        if (three && IN(R, 4, hz) && IN(C, 4, hx)) {
          REAL b2 = IN(Y + 2, 4, ny) ? AT(by, R, Y + 2, C) : (REAL)0;
          REAL b3 = IN(Y + 3, 4, ny) ? AT(by, R, Y + 3, C) : (REAL)0;
          avy = (b2 + b3) * (REAL)0.5;
        }
        const size_t gi = ((size_t)(C - 1) * ny + (Y - 1)) * nz + (R - 1);
        REAL gv = gR[gi] - avx;
        if (three) gv = gv - avy;
        gR[gi] = gv - avz;
      }
#undef IN
}


static void compute_gradient(ctx *c, REAL *gK, REAL *gR, REAL *g3) {
  if (c->d.physics == GPO_ELASTIC) {
    compute_gradient_elastic(c, gK, gR, g3, c->srcamt);
    return;
  }
  const int h = c->h;
  const REAL dtI = c->dtI;
  arr p1 = c->w[0][GPO_P], p1p = c->wp[0][GPO_P], p2p = c->wp[1][GPO_P];
  /* compute_gmodKI!: g += pa_prev * (pf_prev - pf) * dtI */
  for (size_t i = 0; i < alen(p1); i++) gK[i] = gK[i] + p2p.a[i] * (p1p.a[i] - p1.a[i]) * dtI;
  /* compute_gmodrho!: buffer = va_prev * (vf - vf_prev) * dtI */
  const int three = c->d.ndim == 3;
  const int vids[3] = {GPO_VX, GPO_VZ, GPO_VY};
  for (int q = 0; q < 2 + three; q++) {
    arr vf = c->w[0][vids[q]], vfp = c->wp[0][vids[q]], vap = c->wp[1][vids[q]], bf = c->vbuf[q];
    for (size_t i = 0; i < alen(vf); i++) bf.a[i] = vap.a[i] * (vf.a[i] - vfp.a[i]) * dtI;
  }
  if (c->imaging) {
    rho_gather(c, gR);
    return;
  }
  /* combine_gmodrho!: @inn(g) = @inn(g) - @av_xi(vxbuf) - @av_zi(vzbuf).
   * 3-D (no reference counterpart): the same with the y average between
   * them, g - avx - avy - avz, each average one cell off the stencil centre
   * along its axis as in 2-D. */
  arr g;
  g.a = gR;
  g.n1 = c->d.nz;
  g.n2 = c->d.ny;
  g.n3 = c->d.nx;
  arr bx = c->vbuf[0], bz = c->vbuf[1], by = c->vbuf[2];
  const int hy = three ? h : 0;
  for (int ix = 1; ix <= g.n3 - 2 * h; ix++)
    for (int iy = 1; iy <= g.n2 - 2 * hy; iy++)
      for (int iz = 1; iz <= g.n1 - 2 * h; iz++) {
        REAL avx = (AT(bx, iz + h, iy + hy, ix) + AT(bx, iz + h, iy + hy, ix + 1)) * (REAL)0.5;
        REAL avz = (AT(bz, iz, iy + hy, ix + h) + AT(bz, iz + 1, iy + hy, ix + h)) * (REAL)0.5;
        REAL gv = AT(g, iz + h, iy + hy, ix + h) - avx;
        if (three) gv = gv - (AT(by, iz + h, iy, ix + h) + AT(by, iz + h, iy + 1, ix + h)) * (REAL)0.5;
        AT(g, iz + h, iy + hy, ix + h) = gv - avz;
      }
}

/* imaging condition of the discrete elastic scheme (gpo.h, GPO_ADJOINT_HIST).
 * A: the amounts dtM pv the forward step added to every normal stress of a
 * cell (explosive sources), or NULL.  There the stress decrease is K e - A 1
 * instead of K e, and dtM multiplies the source too, so the normal terms
 * gain (sum a)(d A / (dtM + (d-1) dtl) - A / dtM) dtl^2 / dt and
 * (sum a)(A / (dtM + (d-1) dtl) - A / dtM) 2 dt / invmu^2, added first. */
static void compute_gradient_elastic(ctx *c, REAL *gL, REAL *gM, REAL *gR, const REAL *A) {
  const int three = c->d.ndim == 3, h = c->h;
  const REAL dt = c->dt, dtI = c->dtI;
  arr M = c->dmod[c->ndmod - 2], L = c->dmod[c->ndmod - 1], imu = c->mod[1];
  const int nid3[3] = {GPO_TAUXX, GPO_TAUYY, GPO_TAUZZ}, nid2[2] = {GPO_TAUXX, GPO_TAUZZ};
  const int *nid = three ? nid3 : nid2;
  const int d = three ? 3 : 2;
  const size_t n = alen(c->w[0][GPO_TAUXX]);
  for (size_t i = 0; A && i < n; i++) {
    if (A[i] == (REAL)0) continue;
    REAL sq = 0;
    for (int k = 0; k < d; k++) sq = sq + c->wp[1][nid[k]].a[i];
    const REAL beta = L.a[i], alpha = M.a[i] - L.a[i];
    const REAL sa = sq / (alpha + (REAL)d * beta); /* sum of K^-1 q */
    const REAL corr = A[i] / (alpha + (REAL)d * beta), own = A[i] / M.a[i];
    gL[i] = gL[i] + sa * ((REAL)d * corr - own) * (beta * beta * dtI);
    gM[i] = gM[i] + sa * (corr - own) * ((REAL)2 * dt / (imu.a[i] * imu.a[i]));
  }
  for (size_t i = 0; i < n; i++) {
    REAL q[3], dT[3], a[3], b[3], sq = 0, sT = 0;
    for (int k = 0; k < d; k++) {
      q[k] = c->wp[1][nid[k]].a[i];
      dT[k] = c->wp[0][nid[k]].a[i] - c->w[0][nid[k]].a[i];
      sq = sq + q[k];
      sT = sT + dT[k];
    }
    const REAL beta = L.a[i], alpha = M.a[i] - L.a[i];
    const REAL cq = beta / (alpha + (REAL)d * beta);
    REAL sa = 0, sb = 0, ab = 0;
    for (int k = 0; k < d; k++) {
      a[k] = (q[k] - cq * sq) / alpha;
      b[k] = (dT[k] - cq * sT) / alpha;
      sa = sa + a[k];
      sb = sb + b[k];
      ab = ab + a[k] * b[k];
    }
    gL[i] = gL[i] + sa * sb * (beta * beta * dtI);
    gM[i] = gM[i] + ab * ((REAL)2 * dt / (imu.a[i] * imu.a[i]));
  }
  /* shear cells: a quarter of q_s dT_s / dt to each invmu cell of the
   * cell's average (store_invav4) */
  arr g;
  g.a = gM;
  g.n1 = c->d.nz;
  g.n2 = three ? c->d.ny : 1;
  g.n3 = c->d.nx;
  const int sid[3] = {GPO_TAUXZ, GPO_TAUXY, GPO_TAUYZ};
  for (int k = 0; k < (three ? 3 : 1); k++) {
    arr qa = c->wp[1][sid[k]], t0 = c->wp[0][sid[k]], t1 = c->w[0][sid[k]];
    for (int ix = 1; ix <= qa.n3; ix++)
      for (int iy = 1; iy <= qa.n2; iy++)
        for (int iz = 1; iz <= qa.n1; iz++) {
          const REAL v = AT(qa, iz, iy, ix) * (AT(t0, iz, iy, ix) - AT(t1, iz, iy, ix)) * dtI * (REAL)0.25;
          /* the four cells (z, y, x) of the average and the two axes it spans */
          int z = iz, y = iy, x = ix, a1 = 0, a2 = 2; /* z and x */
          if (three && k == 0) y = iy + h;                 /* @av_xzi */
          if (three && k == 1) z = iz + h, a1 = 1, a2 = 2; /* @av_xyi: y and x */
          if (three && k == 2) x = ix + h, a1 = 0, a2 = 1; /* @av_yzi: z and y */
          for (int u = 0; u < 2; u++)
            for (int w = 0; w < 2; w++) {
              int zz = z, yy = y, xx = x;
              if (a1 == 0) zz += u; else yy += u;
              if (a2 == 2) xx += w; else yy += w;
              AT(g, zz, yy, xx) = AT(g, zz, yy, xx) + v;
            }
        }
  }
  /* rho: the velocity terms of the discrete model (gpo_set_imaging 1) */
  const int vids[3] = {GPO_VX, GPO_VZ, GPO_VY};
  for (int q = 0; q < 2 + three; q++) {
    arr vf = c->w[0][vids[q]], vfp = c->wp[0][vids[q]], vap = c->wp[1][vids[q]], bf = c->vbuf[q];
    for (size_t i = 0; i < alen(vf); i++) bf.a[i] = vap.a[i] * (vf.a[i] - vfp.a[i]) * dtI;
  }
  rho_gather(c, gR);
}

static void save_tp(ctx *c, int ipw);

/* forward history (GPO_FORWARD_HIST): slot s holds the stresses (p) after
 * step s and the velocities after step s (s = nt + 1: after the extra half
 * step) */
static int is_stress_field(int f) { return f == GPO_P || f >= GPO_TAUXX; }
static void hist_io(ctx *c, int ishot, int s, int dir, int with_p) {
  REAL *b = c->hist[ishot] + (size_t)s * c->hstep;
  for (int q = 0; q < GPO_NFIELD; q++) {
    if (!c->present[q]) continue;
    arr f = c->w[0][q];
    if (!is_stress_field(q) || with_p) {
      if (dir == 0)
        memcpy(b, f.a, alen(f) * sizeof(REAL));
      else
        memcpy(f.a, b, alen(f) * sizeof(REAL));
    }
    b += alen(f);
  }
}
/* wavefield 1 of adjoint step it from the history: tp = (-p_s, v_{s+1}),
 * t = (-p_{s-1}, v_s) with s = nt - it + 1, as the time-reversed run holds
 * them (p reversed in sign, velocities not) */
static void negate_stresses(ctx *c) {
  for (int q = 0; q < GPO_NFIELD; q++)
    if (c->present[q] && is_stress_field(q)) {
      arr f = c->w[0][q];
      for (size_t i = 0; i < alen(f); i++) f.a[i] = -f.a[i];
    }
}
static void hist_states(ctx *c, int ishot, int it) {
  const int s = c->d.nt - it + 1;
  hist_io(c, ishot, s, 1, 1);
  negate_stresses(c);
  hist_io(c, ishot, s + 1, 1, 0);
  save_tp(c, 0);
  hist_io(c, ishot, s - 1, 1, 1);
  negate_stresses(c);
  hist_io(c, ishot, s, 1, 0);
}

/* ------------------------------------------------------------------ */
/* public API                                                          */
/* ------------------------------------------------------------------ */
static void present_fields(ctx *c) {
  memset(c->present, 0, sizeof(c->present));
  const int three = c->d.ndim == 3;
  c->present[GPO_VX] = c->present[GPO_VZ] = 1;
  if (three) c->present[GPO_VY] = 1;
  if (c->d.physics == GPO_ACOUSTIC)
    c->present[GPO_P] = 1;
  else {
    c->present[GPO_TAUXX] = c->present[GPO_TAUZZ] = c->present[GPO_TAUXZ] = 1;
    if (three) c->present[GPO_TAUYY] = c->present[GPO_TAUXY] = c->present[GPO_TAUYZ] = 1;
  }
}

static arr field_arr(const ctx *c, int f) {
  int kz = FKIND[f][0], ky = FKIND[f][1], kx = FKIND[f][2];
  if (c->d.ndim == 2) ky = KF;
  return mkarr(c, kz, ky, kx);
}

gpo_ctx *SFX(gpo_create)(const gpo_desc *d, const void *const *mod, const void *const *pml, int nshots) {
  ctx *c = (ctx *)calloc(1, sizeof(ctx));
  c->d = *d;
  if (c->d.ndim == 2) c->d.ny = 1;
  c->h = d->order - 1;
  c->hy = d->ndim == 3 ? c->h : 0;
  /* get_fc (src/fdtd/fdtd.jl:313-332): FP64 then converted to Data.Number */
  double den = d->order == 4 ? 24.0 : d->order == 6 ? 1920.0 : d->order == 8 ? 107520.0 : 1.0;
  c->dt = (REAL)d->dt;
  c->dtI = (REAL)(1.0 / d->dt);
  c->dzI = (REAL)(1.0 / (d->dz * den));
  c->dyI = (REAL)(1.0 / (d->dy * den));
  c->dxI = (REAL)(1.0 / (d->dx * den));
  if (d->physics == GPO_ACOUSTIC) {
    c->ds = d->ndim == 2 ? DA2 : DA3;
    c->nder = d->ndim == 2 ? 4 : 6;
    c->nmod = 2;
  } else {
    c->ds = d->ndim == 2 ? DE2 : DE3;
    c->nder = d->ndim == 2 ? 8 : 18;
    c->nmod = 3;
  }
  for (int i = 0; i < c->nmod; i++) {
    c->mod[i] = mkarr(c, KF, KF, KF);
    memcpy(c->mod[i].a, mod[i], alen(c->mod[i]) * sizeof(REAL));
  }
  for (int q = 0; q < c->nder; q++) {
    size_t n = 2 * (size_t)d->npml;
    c->pa[q] = (REAL *)malloc(n * sizeof(REAL));
    c->pb[q] = (REAL *)malloc(n * sizeof(REAL));
    c->pk[q] = (REAL *)malloc(n * sizeof(REAL));
    memcpy(c->pa[q], pml[3 * q + 0], n * sizeof(REAL));
    memcpy(c->pb[q], pml[3 * q + 1], n * sizeof(REAL));
    memcpy(c->pk[q], pml[3 * q + 2], n * sizeof(REAL));
  }
  update_dmod(c);
  present_fields(c);
  size_t maxlen = 0;
  for (int ipw = 0; ipw < 2; ipw++) {
    for (int f = 0; f < GPO_NFIELD; f++) {
      if (!c->present[f]) continue;
      c->w[ipw][f] = field_arr(c, f);
      c->wp[ipw][f] = field_arr(c, f);
      if (alen(c->w[ipw][f]) > maxlen) maxlen = alen(c->w[ipw][f]);
    }
    for (int q = 0; q < c->nder; q++) {
      const dspec *s = &c->ds[q];
      c->der[ipw][q] = mkarr(c, s->kz, s->ky, s->kx);
      arr m = mkarr(c, s->kz, s->ky, s->kx); /* then the axis set to 2*npml */
      free(m.a);
      if (s->axis == 0) m.n1 = 2 * d->npml;
      if (s->axis == 1) m.n2 = 2 * d->npml;
      if (s->axis == 2) m.n3 = 2 * d->npml;
      m.a = (REAL *)calloc(alen(m), sizeof(REAL));
      c->mem[ipw][q] = m;
    }
  }
  c->vbuf[0] = field_arr(c, GPO_VX);
  c->vbuf[1] = field_arr(c, GPO_VZ);
  if (d->ndim == 3) c->vbuf[2] = field_arr(c, GPO_VY);
  c->hstep = 0;
  for (int f = 0; f < GPO_NFIELD; f++)
    if (c->present[f]) c->hstep += alen(c->w[0][f]);
  c->pvlen = maxlen;
  c->pv = (REAL *)calloc(maxlen, sizeof(REAL));
  c->pvflag = (unsigned char *)calloc(maxlen, 1);
  /* boundary store: per step the strips of the saved stress fields, then the
   * final snapshots of the saved stress fields and the velocities. */
  int ids[3];
  const int ns = nsaved(c, ids);
  c->bstep = 0;
  c->bsnap = 0;
  for (int q = 0; q < ns; q++) {
    arr f = c->w[0][ids[q]];
    for (int axis = 0; axis < 3; axis++)
      if (!(axis == 1 && d->ndim == 2)) c->bstep += strip_len(c, f, axis);
    c->bsnap += alen(f);
  }
  c->bsnap += alen(c->w[0][GPO_VX]) + alen(c->w[0][GPO_VZ]);
  if (d->ndim == 3) c->bsnap += alen(c->w[0][GPO_VY]);
  c->nshots = nshots;
  c->bstore = (REAL **)calloc((size_t)nshots, sizeof(REAL *));
  c->hist = (REAL **)calloc((size_t)nshots, sizeof(REAL *));
  c->snaps = (REAL **)calloc((size_t)nshots, sizeof(REAL *));
  c->illum = (double **)calloc((size_t)nshots, sizeof(double *));
  c->snap_field = -1;
  return (gpo_ctx *)c;
}

static void reset_w(ctx *c) {
  /* reset_w2! (src/fdtd/types.jl:101-113) */
  for (int ipw = 0; ipw < 2; ipw++) {
    for (int f = 0; f < GPO_NFIELD; f++)
      if (c->present[f]) {
        azero(c->w[ipw][f]);
        azero(c->wp[ipw][f]);
      }
    for (int q = 0; q < c->nder; q++) {
      azero(c->der[ipw][q]);
      azero(c->mem[ipw][q]);
    }
  }
}

static void save_tp(ctx *c, int ipw) {
  for (int f = 0; f < GPO_NFIELD; f++)
    if (c->present[f]) acopy(c->wp[ipw][f], c->w[ipw][f]);
}

/* Born secondary source: dst += r * (now - prev) (GPO_BORN) */
static void born_add(arr dst, arr r, arr now, arr prev) {
  for (size_t i = 0; i < alen(dst); i++) dst.a[i] = dst.a[i] + r.a[i] * (now.a[i] - prev.a[i]);
}


/* mod_x_proc! for one supersource (src/fdtd/propagate.jl:138-261) */
int SFX(gpo_shot)(gpo_ctx *cc, int ishot, int mode, int nsrc, const gpo_proj *src, int nrec, gpo_proj *rec,
                  int nadj, const gpo_proj *adj, void *grad_invK, void *grad_rho, void *grad_3) {
  ctx *c = (ctx *)cc;
  if (ishot < 0 || ishot >= c->nshots) return -1;
#ifdef _OPENMP
  if (c->d.nthreads > 0) omp_set_num_threads(c->d.nthreads);
#endif
  const int nt = c->d.nt;
  const int hist = mode == GPO_FORWARD_HIST || mode == GPO_ADJOINT_HIST;
  const int adjoint = mode == GPO_ADJOINT || mode == GPO_ADJOINT_HIST;
  if ((mode == GPO_FORWARD_SAVE || mode == GPO_ADJOINT) && !c->bstore[ishot])
    c->bstore[ishot] = (REAL *)calloc((size_t)nt * c->bstep + c->bsnap, sizeof(REAL));
  if (hist && c->d.physics != GPO_ACOUSTIC && (c->d.free_faces & GPO_ZMIN)) return -2;
  if (mode == GPO_FORWARD_HIST && !c->hist[ishot])
    c->hist[ishot] = (REAL *)calloc((size_t)(nt + 2) * c->hstep, sizeof(REAL));
  if (mode == GPO_ADJOINT_HIST && !c->hist[ishot]) return -3;
  if (mode == GPO_ADJOINT && (c->d.physics != GPO_ACOUSTIC || c->d.ndim != 2) && (grad_invK || grad_rho)) return -2;
  const int born = mode == GPO_BORN;
  if (born && !c->have_born) return -4;
  reset_w(c);
  /* initialize! (types.jl:67-72): the illumination of this run */
  if (c->illum_on) {
    if (!c->illum[ishot]) c->illum[ishot] = (double *)malloc(alen(c->w[0][GPO_P]) * sizeof(double));
    for (size_t i = 0; i < alen(c->w[0][GPO_P]); i++) c->illum[ishot][i] = 0.0;
  }
  if (mode == GPO_ADJOINT) {
    snap_io(c, ishot, 1, 1); /* boundary_force_snap_tau! */
    snap_io(c, ishot, 0, 1); /* boundary_force_snap_v! */
  }
  /* the history run propagates the adjoint wavefield alone */
  const int pw0 = mode == GPO_ADJOINT_HIST ? 1 : 0;
  const int npw = adjoint || born ? 2 : 1;
  /* the records of a Born run are wavefield 2's */
  arr *wr = born ? c->w[1] : c->w[0];
  const int vids3[3] = {GPO_VX, GPO_VY, GPO_VZ};
  for (int it = 1; it <= nt; it++) {
    /* record! [:p] */
    for (int r = 0; r < nrec; r++)
      if (rec[r].field == GPO_P) record(c, wr, &rec[r], it - 1);
    if (born) {
      save_tp(c, 0);
      for (int ipw = 0; ipw < 2; ipw++) update_dstress(c, ipw);
      update_v(c, 0);
      for (int s = 0; s < nsrc; s++)
        if (is_velocity(src[s].field)) add_velocity_source(c, c->w[0], &src[s], it - 1);
      /* velocity secondary sources, then wavefield 2's own update */
      for (int q = 0; q < 3; q++)
        if (c->present[vids3[q]])
          born_add(c->w[1][vids3[q]], c->born[q + 1], c->w[0][vids3[q]], c->wp[0][vids3[q]]);
      update_v(c, 1);
      for (int r = 0; r < nrec; r++)
        if (is_velocity(rec[r].field)) record(c, wr, &rec[r], it - 1);
      for (int ipw = 0; ipw < 2; ipw++) update_dv(c, ipw);
      for (int ipw = 0; ipw < 2; ipw++) update_stress(c, ipw);
      for (int s = 0; s < nsrc; s++)
        if (is_stress_src(src[s].field)) add_stress_source(c, c->w[0], &src[s], it - 1);
      born_add(c->w[1][GPO_P], c->born[0], c->w[0][GPO_P], c->wp[0][GPO_P]);
      continue;
    }
    if (mode == GPO_ADJOINT) {
      save_tp(c, 0);
      save_tp(c, 1);
      boundary_force(c, ishot, nt - it + 1);
    }
    if (mode == GPO_ADJOINT_HIST) {
      save_tp(c, 1);
      hist_states(c, ishot, it);
      if (c->d.physics == GPO_ELASTIC) {
        /* the amounts dtM pv the forward step s = nt - it + 1 added to the
         * normal stresses (add_stress_source!, wavelet sample s - 1) */
        const size_t n = alen(c->w[0][GPO_TAUXX]);
        if (!c->srcamt) c->srcamt = (REAL *)calloc(n, sizeof(REAL));
        memset(c->srcamt, 0, n * sizeof(REAL));
        arr dM = c->dmod[c->ndmod - 2];
        for (int s = 0; s < nsrc; s++) {
          if (!is_stress_src(src[s].field)) continue;
          spray(c, &src[s], nt - it);
          for (int j = 0; j < src[s].n; j++)
            for (int64_t k = src[s].colptr[j]; k < src[s].colptr[j + 1]; k++) {
              const int64_t r = src[s].rowval[k];
              if (c->pvflag[r] == 1) continue;
              c->pvflag[r] = 1;
              c->srcamt[r] = c->srcamt[r] + c->pv[r] * dM.a[r];
            }
          spray_clear(c, &src[s]);
        }
      }
    }
    for (int ipw = pw0; ipw < npw; ipw++) update_dstress(c, ipw);
    for (int ipw = pw0; ipw < npw; ipw++) update_v(c, ipw);
    /* add_velocity_source! (wavefield 1, then the adjoint wavefield) */
    for (int s = 0; s < nsrc && !pw0; s++)
      if (is_velocity(src[s].field)) add_velocity_source(c, c->w[0], &src[s], it - 1);
    if (adjoint)
      for (int s = 0; s < nadj; s++)
        if (is_velocity(adj[s].field)) add_velocity_source(c, c->w[1], &adj[s], it - 1);
    /* record! [:vx, :vy, :vz] */
    for (int r = 0; r < nrec; r++)
      if (is_velocity(rec[r].field)) record(c, c->w[0], &rec[r], it - 1);
    for (int ipw = pw0; ipw < npw; ipw++) update_dv(c, ipw);
    for (int ipw = pw0; ipw < npw; ipw++) update_stress(c, ipw);
    /* add_stress_source! (wavefield 1 only) */
    for (int s = 0; s < nsrc && !pw0; s++)
      if (is_stress_src(src[s].field)) add_stress_source(c, c->w[0], &src[s], it - 1);
    if (mode == GPO_FORWARD_SAVE) boundary_save(c, ishot, it);
    if (mode == GPO_FORWARD_HIST) hist_io(c, ishot, it, 0, 1);
    if (adjoint && (grad_invK || grad_rho)) compute_gradient(c, (REAL *)grad_invK, (REAL *)grad_rho, (REAL *)grad_3);
    /* compute_illum! (propagate.jl:236, commented out in the reference):
       illum[i] += abs2(p[i]), the square in the field's precision */
    if (c->illum_on) {
      const REAL *p = c->w[0][GPO_P].a;
      for (size_t i = 0; i < alen(c->w[0][GPO_P]); i++) {
        const REAL v = p[i] * p[i];
        c->illum[ishot][i] += (double)v;
      }
    }
    /* snaps_save! for wavefield 1 at the end of step it (propagate.jl:238-245) */
    for (int k = 0; k < c->nsnap; k++)
      if (c->snap_its[k] == it) {
        arr f = c->w[0][c->snap_field];
        if (!c->snaps[ishot]) c->snaps[ishot] = (REAL *)calloc((size_t)c->nsnap * alen(f), sizeof(REAL));
        memcpy(c->snaps[ishot] + (size_t)k * alen(f), f.a, alen(f) * sizeof(REAL));
      }
  }
  if (mode == GPO_ADJOINT_HIST || born) return 0;
  if (mode == GPO_FORWARD_SAVE) snap_io(c, ishot, 1, 0); /* boundary_save_snap_tau! */
  update_dstress(c, 0);
  update_v(c, 0);
  if (mode == GPO_FORWARD_SAVE) snap_io(c, ishot, 0, 0); /* boundary_save_snap_v! */
  if (mode == GPO_FORWARD_HIST) hist_io(c, ishot, nt + 1, 0, 0);
  return 0;
}

/* Born secondary-source ratios (see GPO_BORN): rp on the p grid, rv on each
 * velocity grid over its update domain (store_invav: velocity cell i along
 * an axis averages rho at i-3 and i-2) */
int SFX(gpo_set_born)(gpo_ctx *cc, const void *dinvK, const void *drho) {
  ctx *c = (ctx *)cc;
  if (c->d.physics != GPO_ACOUSTIC) return -1;
  const REAL *dK = (const REAL *)dinvK, *dR = (const REAL *)drho;
  const int three = c->d.ndim == 3, h = c->h, hy = c->hy;
  const int ids[4] = {GPO_P, GPO_VX, GPO_VY, GPO_VZ};
  for (int q = 0; q < 4; q++) {
    if (!c->present[ids[q]]) continue;
    if (!c->have_born) c->born[q] = field_arr(c, ids[q]);
    azero(c->born[q]);
  }
  arr rho = c->mod[1], K = c->mod[0];
  const int nz = c->d.nz, ny = three ? c->d.ny : 1, nx = c->d.nx;
  for (int C = 1; C <= nx; C++)
    for (int Y = 1; Y <= ny; Y++)
      for (int R = 1; R <= nz; R++) {
        const size_t i = ((size_t)(C - 1) * ny + (Y - 1)) * nz + (R - 1);
        AT(c->born[0], R, Y, C) = -(dK[i] / K.a[i]);
      }
  /* velocity cells: (axis offset along the velocity's own axis) */
  const int vq[3] = {1, 2, 3}; /* born index of vx, vy, vz */
  for (int q = 0; q < 3; q++) {
    if (q == 1 && !three) continue;
    arr v = c->born[vq[q]];
    const int ax = q == 0 ? 2 : q == 1 ? 1 : 0; /* x, y, z */
    const int r1 = v.n1 - 2 * h, r2 = three ? v.n2 - 2 * hy : 1, r3 = v.n3 - 2 * h;
    for (int ix = 1; ix <= r3; ix++)
      for (int iy = 1; iy <= r2; iy++)
        for (int iz = 1; iz <= r1; iz++) {
          const int R = iz + h, Y = three ? iy + hy : 1, C = ix + h;
          /* density cells of the coefficient (store_invav) */
          int za = R, ya = Y, xa = C;
          if (ax == 0) za = R - h;
          if (ax == 1) ya = Y - h;
          if (ax == 2) xa = C - h;
          const int zb = za + (ax == 0), yb = ya + (ax == 1), xb = xa + (ax == 2);
          const size_t ia = ((size_t)(xa - 1) * ny + (ya - 1)) * nz + (za - 1);
          const size_t ib = ((size_t)(xb - 1) * ny + (yb - 1)) * nz + (zb - 1);
          AT(v, R, Y, C) = -((dR[ia] + dR[ib]) / (rho.a[ia] + rho.a[ib]));
        }
  }
  c->have_born = 1;
  return 0;
}

int SFX(gpo_set_imaging)(gpo_ctx *cc, int mode) {
  ctx *c = (ctx *)cc;
  if (mode < 0 || mode > 1) return -1;
  c->imaging = mode;
  return 0;
}

int SFX(gpo_set_snaps)(gpo_ctx *cc, int field, int n, const int *its) {
  ctx *c = (ctx *)cc;
  if (n < 0 || n > 64 || (n > 0 && (field < 0 || field >= GPO_NFIELD || !c->present[field]))) return -1;
  c->snap_field = field;
  c->nsnap = n;
  for (int k = 0; k < n; k++) c->snap_its[k] = its[k];
  return 0;
}

int SFX(gpo_set_illum)(gpo_ctx *cc, int on) {
  ctx *c = (ctx *)cc;
  if (on && !c->present[GPO_P]) return -1;
  c->illum_on = on != 0;
  return 0;
}

/* the illumination of shot ishot's last run over the p array (extended) */
int SFX(gpo_get_illum)(gpo_ctx *cc, int ishot, double *out) {
  ctx *c = (ctx *)cc;
  if (ishot < 0 || ishot >= c->nshots || !c->illum[ishot]) return -1;
  memcpy(out, c->illum[ishot], alen(c->w[0][GPO_P]) * sizeof(double));
  return 0;
}

int SFX(gpo_get_snap)(gpo_ctx *cc, int ishot, int k, void *out) {
  ctx *c = (ctx *)cc;
  if (ishot < 0 || ishot >= c->nshots || k < 0 || k >= c->nsnap || !c->snaps[ishot]) return -1;
  arr f = c->w[0][c->snap_field];
  memcpy(out, c->snaps[ishot] + (size_t)k * alen(f), alen(f) * sizeof(REAL));
  return 0;
}

int SFX(gpo_get_field)(gpo_ctx *cc, int ipw, int field, void *out) {
  ctx *c = (ctx *)cc;
  if (field < 0 || field >= GPO_NFIELD || !c->present[field] || ipw < 1 || ipw > 2) return -1;
  arr f = c->w[ipw - 1][field];
  memcpy(out, f.a, alen(f) * sizeof(REAL));
  return 0;
}

void SFX(gpo_destroy)(gpo_ctx *cc) {
  ctx *c = (ctx *)cc;
  if (!c) return;
  for (int i = 0; i < c->nmod; i++) free(c->mod[i].a);
  for (int i = 0; i < c->ndmod; i++) free(c->dmod[i].a);
  for (int q = 0; q < c->nder; q++) {
    free(c->pa[q]);
    free(c->pb[q]);
    free(c->pk[q]);
  }
  for (int ipw = 0; ipw < 2; ipw++) {
    for (int f = 0; f < GPO_NFIELD; f++) {
      free(c->w[ipw][f].a);
      free(c->wp[ipw][f].a);
    }
    for (int q = 0; q < c->nder; q++) {
      free(c->der[ipw][q].a);
      free(c->mem[ipw][q].a);
    }
  }
  for (int q = 0; q < 4; q++) free(c->born[q].a);
  free(c->srcamt);
  free(c->vbuf[0].a);
  free(c->vbuf[1].a);
  free(c->vbuf[2].a);
  for (int i = 0; i < c->nshots; i++) free(c->hist[i]);
  free(c->hist);
  for (int i = 0; i < c->nshots; i++) free(c->snaps[i]);
  free(c->snaps);
  for (int i = 0; i < c->nshots; i++) free(c->illum[i]);
  free(c->illum);
  free(c->pv);
  free(c->pvflag);
  for (int i = 0; i < c->nshots; i++) free(c->bstore[i]);
  free(c->bstore);
  free(c);
}

int SFX(gpo_get_dmod)(gpo_ctx *cc, int idx, void *out, int *n1, int *n2, int *n3) {
  ctx *c = (ctx *)cc;
  if (idx < 0 || idx >= c->ndmod) return -1;
  arr f = c->dmod[idx];
  *n1 = f.n1;
  *n2 = f.n2;
  *n3 = f.n3;
  if (out) memcpy(out, f.a, alen(f) * sizeof(REAL));
  return 0;
}

#ifdef GPO_PRIMARY
int gpo_field_shape(const gpo_desc *d, int field, int *n1, int *n2, int *n3) {
  ctx c;
  memset(&c, 0, sizeof(c));
  c.d = *d;
  if (c.d.ndim == 2) c.d.ny = 1;
  c.h = d->order - 1;
  if (field < 0 || field >= GPO_NFIELD) return -1;
  int ky = d->ndim == 2 ? KF : FKIND[field][1];
  *n1 = nk(&c, FKIND[field][0], c.d.nz, 1);
  *n2 = nk(&c, ky, c.d.ny, d->ndim == 3);
  *n3 = nk(&c, FKIND[field][2], c.d.nx, 1);
  return 0;
}
#endif
