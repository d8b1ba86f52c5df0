/*
 * gpo.h -- interface of the CPU ORACLE for the GeoPhyInv FDTD hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a literal CPU restatement of the
 * reference's staggered-grid time loop (src/fdtd/propagate.jl:138-261 and
 * the kernels it calls).  It is the checker for the CUDA implementation and
 * the timed CPU baseline; nothing in the product links or calls it.
 *
 * Parity status: the reference is Julia and cannot run in this environment,
 * and its test suite ships no golden vectors.  The oracle is pinned by the
 * reference's own property / known-answer tests restated in tests/ (the
 * time-reversal test test/fdtd/backprop.jl:7-47 and the analytic Green's
 * function test test/fdtd/accuracy2D.jl:6-82), not by outputs of the
 * reference itself: "parity unpinned" in the sense of bit-level reference
 * outputs.
 *
 * Conventions (mirroring the reference):
 *   - arrays are column-major with z fastest, 1-based in the comments;
 *   - a 2-D run is a 3-D run with ny = 1 and no y stencils;
 *   - the "extended" grid (nz, ny, nx) already contains the PML padding;
 *   - field shapes follow get_mgrid (src/fields.jl:92-671).
 */
#ifndef GPO_H
#define GPO_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { GPO_ACOUSTIC = 0, GPO_ELASTIC = 1 };
enum { GPO_FORWARD = 0, GPO_FORWARD_SAVE = 1, GPO_ADJOINT = 2, GPO_FORWARD_HIST = 3, GPO_ADJOINT_HIST = 4,
       GPO_BORN = 5 };
/* GPO_BORN (acoustic, after gpo_set_born): linearised (Born) modelling.
 * Wavefield 1 is the background run; wavefield 2 runs the same scheme with
 * no sources of its own, driven by the secondary sources of the
 * perturbation: after wavefield 1's velocity update, each velocity cell of
 * wavefield 2 gains rv * (v1 - v1_prev) (before its own update), and after
 * the stress update each p cell gains rp * (p1 - p1_prev), with
 * rv = -(drho_a + drho_b) / (rho_a + rho_b) over the two density cells of
 * the cell's update coefficient and rp = -dinvK / invK.  The records are
 * wavefield 2's.  This is the exact linearisation of the discrete scheme
 * in the medium parameters (no reference counterpart: the reference's
 * born.jl passes arguments its kernels do not take). */
/* GPO_FORWARD_HIST / GPO_ADJOINT_HIST (acoustic, 2-D and 3-D): the same
 * gradient as forward_save -> adjoint, but wavefield 1 is not rebuilt by
 * time reversal: the forward run keeps its whole history (p and v after
 * every step, and v after the extra half step) and the adjoint run takes
 * wavefield 1's old and new states from it.  This is the gradient that a
 * checkpointed adjoint computes (forward states recomputed, not reversed). */
/* face bits, in the reference's naming (:zmin, :zmax, :ymin, ...) */
enum { GPO_ZMIN = 1, GPO_ZMAX = 2, GPO_YMIN = 4, GPO_YMAX = 8, GPO_XMIN = 16, GPO_XMAX = 32 };
/* wavefield ids (the reference's Fields symbols, non-derivative part) */
enum {
  GPO_P = 0, GPO_VX = 1, GPO_VY = 2, GPO_VZ = 3,
  GPO_TAUXX = 4, GPO_TAUYY = 5, GPO_TAUZZ = 6,
  GPO_TAUXY = 7, GPO_TAUXZ = 8, GPO_TAUYZ = 9, GPO_NFIELD = 10
};

typedef struct {
  int physics;       /* GPO_ACOUSTIC / GPO_ELASTIC */
  int ndim;          /* 2 or 3 */
  int order;         /* 2, 4, 6, 8 (_fd_order) */
  int nz, ny, nx;    /* extended grid; ny = 1 in 2-D */
  int npml;          /* _fd_npml = 40 + order - 1 */
  int nbound;        /* _fd_nbound = 3 */
  int pml_faces;     /* bit mask of PML faces */
  int rigid_faces;   /* rigid faces (the reference stores rigid U pml) */
  int free_faces;    /* stress-free faces (zmin only is honoured) */
  int nt;
  int nthreads;      /* OpenMP threads, <= 0: library default */
  double dt, dz, dy, dx;
} gpo_desc;

/* A sparse projection (CSC, 0-based) between one field's grid and n
 * sources or receivers, with its n time series (nt x n, column-major). */
typedef struct {
  int field;               /* GPO_P ... */
  int n;                   /* columns */
  const int64_t *colptr;   /* n + 1 */
  const int64_t *rowval;   /* linear index into the field array */
  const void *nzval;       /* REAL weights */
  void *data;              /* REAL nt x n: wavelet (in) or record (out) */
} gpo_proj;

typedef struct gpo_ctx gpo_ctx;

/* mod: acoustic {invK, rho}, elastic {invlambda, invmu, rho} on the extended
 * grid.  pml: for each derivative field in the canonical order below, three
 * arrays a, b, kI of length 2*npml -> 3*nderiv pointers.
 * Canonical derivative order:
 *   acoustic 2-D: dpdx dpdz dvxdx dvzdz
 *   elastic  2-D: dtauxxdx dtauxzdx dtauzzdz dtauxzdz dvxdx dvzdz dvxdz dvzdx
 *   acoustic 3-D: dpdx dpdy dpdz dvxdx dvydy dvzdz
 *   elastic  3-D: dtauxxdx dtauxydx dtauxzdx dtauyydy dtauxydy dtauyzdy
 *                 dtauzzdz dtauyzdz dtauxzdz dvxdx dvydy dvzdz dvxdy dvxdz
 *                 dvydx dvydz dvzdx dvzdy                                  */
gpo_ctx *gpo_create_f32(const gpo_desc *d, const void *const *mod, const void *const *pml, int nshots);
gpo_ctx *gpo_create_f64(const gpo_desc *d, const void *const *mod, const void *const *pml, int nshots);
/* Run one supersource (shot) in the given mode.  rec data are written
 * (records), src/adj data are read.  grad (acoustic adjoint only; 3-D only
 * with GPO_ADJOINT_HIST): two extended-grid arrays {invK, rho} that the
 * shot's gradient is ADDED to. */
int gpo_shot_f32(gpo_ctx *c, int ishot, int mode, int nsrc, const gpo_proj *src, int nrec,
                 gpo_proj *rec, int nadj, const gpo_proj *adj, void *grad_invK, void *grad_rho, void *grad_3);
int gpo_shot_f64(gpo_ctx *c, int ishot, int mode, int nsrc, const gpo_proj *src, int nrec,
                 gpo_proj *rec, int nadj, const gpo_proj *adj, void *grad_invK, void *grad_rho, void *grad_3);
/* Elastic media (GPO_ADJOINT_HIST only, no free surface): the three arrays
 * are the gradients with respect to {invlambda, invmu, rho}, from the
 * imaging condition of the discrete elastic scheme (no reference
 * counterpart: the reference defines gradients for 2-D acoustic media
 * only, src/fdtd/gradient.jl:17-64):
 *   normal-stress cells, with K = (dtM - dtl) I + dtl 1 1' the cell's
 *   stiffness, q the adjoint normal stresses before the adjoint step and
 *   dT the forward normal-stress decrease of the forward step,
 *   a = K^-1 q, b = K^-1 dT:
 *     g_invlambda += (sum a)(sum b) dtl^2 / dt
 *     g_invmu     += (a . b) 2 dt / invmu^2
 *   shear cells: each of the four invmu cells of the cell's average gains
 *     q_s dT_s / (4 dt)
 *   velocity cells: the rho term of gpo_set_imaging mode 1. */
/* Imaging condition of the rho gradient: 0 the reference's
 * (src/fdtd/gradient.jl:31-56); 1 the gradient of the discrete model, over
 * the velocity cells whose update coefficient holds rho (no reference
 * counterpart; checked against finite differences). */
int gpo_set_imaging_f32(gpo_ctx *c, int mode);
/* Perturbations (dinvK, drho) of the medium on the extended grid for
 * GPO_BORN runs (the medium perturbation minus the medium, as
 * update!(pa, medium, medium_pert) forms it, src/fdtd/medium.jl:103-126). */
int gpo_set_born_f32(gpo_ctx *c, const void *dinvK, const void *drho);
int gpo_set_born_f64(gpo_ctx *c, const void *dinvK, const void *drho);
int gpo_set_imaging_f64(gpo_ctx *c, int mode);
/* snaps_save! (src/fdtd/fdtd.jl:586-591): keep wavefield 1's `field` at
 * the end of steps its[0..n) of later shots; read them per shot and k. */
int gpo_set_snaps_f32(gpo_ctx *c, int field, int n, const int *its);
int gpo_set_snaps_f64(gpo_ctx *c, int field, int n, const int *its);
int gpo_get_snap_f32(gpo_ctx *c, int ishot, int k, void *out);
int gpo_get_snap_f64(gpo_ctx *c, int ishot, int k, void *out);
/* illum_flag (src/fdtd/fdtd.jl:571-582): per shot, sum over the steps of
 * p^2 of wavefield 1 (the square in the oracle's precision, the sum in
 * double) over the p array */
int gpo_set_illum_f32(gpo_ctx *c, int on);
int gpo_set_illum_f64(gpo_ctx *c, int on);
int gpo_get_illum_f32(gpo_ctx *c, int ishot, double *out);
int gpo_get_illum_f64(gpo_ctx *c, int ishot, double *out);
/* Copy the current (last shot's final) state of a field of wavefield ipw (1 or 2). */
int gpo_get_field_f32(gpo_ctx *c, int ipw, int field, void *out);
int gpo_get_field_f64(gpo_ctx *c, int ipw, int field, void *out);
/* Shape of a field (n1, n2, n3) for this descriptor. */
int gpo_field_shape(const gpo_desc *d, int field, int *n1, int *n2, int *n3);
/* The dmod arrays (update_dmod!, src/fdtd/medium.jl:143-221) in the order of
 * MediumParameters (src/fdtd/medium.jl:81-95), for cross-checking setup. */
int gpo_get_dmod_f32(gpo_ctx *c, int idx, void *out, int *n1, int *n2, int *n3);
void gpo_destroy_f32(gpo_ctx *c);
void gpo_destroy_f64(gpo_ctx *c);

#ifdef __cplusplus
}
#endif
#endif
