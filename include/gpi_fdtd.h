/*
 * gpi_fdtd.h -- C ABI of the GB300 FDTD engine (libgpi_fdtd.so).
 *
 * The engine replaces the per-worker time loop of GeoPhyInv.jl
 * (mod_x_proc!, src/fdtd/propagate.jl:138-261) and the device-side parts of
 * its setup.  A Julia host keeps SeisForwExpt / update! and reaches the
 * engine through `ccall` on these entry points; every entry point below
 * names the reference function it stands in for.
 *
 * Conventions
 *   - all arrays are column-major (z fastest), like Julia arrays;
 *   - the grid is the EXTENDED grid (physical grid plus PML padding),
 *     exactly pac.exmedium.grid of the reference;
 *   - sparse projections are CSC with 0-based column pointers and 0-based
 *     linear row indices into the field's own array (get_mgrid shapes);
 *   - every call returns 0 on success or a negative GPI_E* code; the
 *     message of the last failure of a plan is gpi_last_error(plan);
 *   - a plan is bound to the CUDA device that was current at creation and
 *     to one stream; calls on one plan are not re-entrant.
 */
#ifndef GPI_FDTD_H
#define GPI_FDTD_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPI_ABI_VERSION 2

enum gpi_status {
  GPI_OK = 0,
  GPI_E_INVALID = -1,     /* bad argument or inconsistent sizes */
  GPI_E_NOMEM = -2,       /* device allocation failed (HBM budget) */
  GPI_E_CUDA = -3,        /* CUDA runtime error */
  GPI_E_UNSUPPORTED = -4, /* combination the engine does not implement */
  GPI_E_STATE = -5        /* call out of order (e.g. adjoint before forward_save) */
};

enum gpi_physics { GPI_ACOUSTIC = 0, GPI_ELASTIC = 1 };
/* GPI_BORN: linearised (Born) modelling, see gpi_set_born */
enum gpi_mode { GPI_FORWARD = 0, GPI_FORWARD_SAVE = 1, GPI_ADJOINT = 2, GPI_BORN = 3 };
/* faces, named as the reference's symbols :zmin, :zmax, :ymin, ... */
enum gpi_face { GPI_ZMIN = 1, GPI_ZMAX = 2, GPI_YMIN = 4, GPI_YMAX = 8, GPI_XMIN = 16, GPI_XMAX = 32 };
/* wavefields (the non-derivative Fields of src/fields.jl:27-42) */
enum gpi_field {
  GPI_P = 0, GPI_VX = 1, GPI_VY = 2, GPI_VZ = 3,
  GPI_TAUXX = 4, GPI_TAUYY = 5, GPI_TAUZZ = 6,
  GPI_TAUXY = 7, GPI_TAUXZ = 8, GPI_TAUYZ = 9
};
/* medium parameters (MediumParameters, src/fdtd/medium.jl:81-95):
 * acoustic {invK, rho}, elastic {invlambda, invmu, rho} */
enum gpi_param { GPI_INVK = 0, GPI_RHO = 1, GPI_INVLAMBDA = 0, GPI_INVMU = 1, GPI_RHO_E = 2 };

typedef struct gpi_plan gpi_plan;

typedef struct {
  int32_t physics;     /* gpi_physics */
  int32_t ndim;        /* 2 or 3 */
  int32_t order;       /* stencil order (_fd_order): 2, 4, 6 or 8; other orders than 4
                          run forward only (npw 1, no checkpoints) */
  int32_t nz, ny, nx;  /* extended grid sizes (ny = 1 for 2-D) */
  int32_t npml;        /* PML width, _fd_npml = 40 + order - 1 */
  int32_t nbound;      /* boundary strip width, _fd_nbound = 3 */
  int32_t pml_faces;   /* gpi_face bit mask */
  int32_t rigid_faces; /* rigid faces; the engine adds pml_faces (fdtd.jl:215) */
  int32_t free_faces;  /* stress-free faces (only GPI_ZMIN is honoured, as in the reference) */
  int32_t nt;          /* time steps */
  int32_t nshots;      /* supersources held by the plan */
  int32_t npw;         /* propagating wavefields: 1 (forward) or 2 (forward_save + adjoint) */
  /* > 0 (acoustic, npw = 2): a checkpointed adjoint instead of the boundary
   * store (boundary.jl): forward_save keeps this many full states of
   * wavefield 1 on the device and the adjoint run recomputes forward states
   * from them on a binomial schedule; 3-D acoustic gradients too.  No
   * counterpart in the reference.  0: the reference's boundary store. */
  int32_t checkpoints;
  /* rho term of the acoustic imaging condition: 0 the reference's
   * (compute_gmodrho!/combine_gmodrho!, src/fdtd/gradient.jl:31-56: the
   * velocity terms averaged 4-5 cells off the cells whose coefficients hold
   * rho); 1 the gradient of the discrete model, rho at (r, c) taking half
   * of the vx terms at columns c+2, c+3 and of the vz terms at rows r+2, r+3
   * (and vy at y+2, y+3) where those cells are updated, which agrees with
   * finite differences.  No counterpart in the reference. */
  int32_t imaging;
  int32_t reserved[2];
  double dt, dz, dy, dx; /* time step and grid steps (dy ignored in 2-D) */
} gpi_plan_desc;

/* PFdtd constructor, device half (src/fdtd/fdtd.jl:61-297, :340-385):
 * allocates wavefields, CPML memory, coefficient arrays, record buffers. */
int gpi_plan_create(const gpi_plan_desc *desc, gpi_plan **out);
/* Frees everything the plan owns (the reference relies on the GC). */
void gpi_plan_destroy(gpi_plan *plan);
/* Message of the last failing call on `plan` (or of the last failing
 * gpi_plan_create when plan is NULL). */
const char *gpi_last_error(const gpi_plan *plan);
/* Run on this CUDA stream (cudaStream_t); NULL is the legacy default stream. */
int gpi_set_stream(gpi_plan *plan, void *stream);
/* Device bytes the plan holds. */
int gpi_plan_bytes(const gpi_plan *plan, size_t *bytes);
/* Device bytes gpi_plan_create would allocate for `desc` (wavefields, CPML
 * memory, coefficients, boundary store or checkpoint slots), computed
 * without allocating; the record buffers (nt x receivers per shot and
 * field) come on top.  No counterpart in the reference; a server admits
 * requests against its HBM budget with it. */
int gpi_plan_estimate(const gpi_plan_desc *desc, size_t *bytes);

/* update!(pac, medium) -> update_dmod! (src/fdtd/medium.jl:131-221):
 * mod[i] is the i-th MediumParameters array on the extended grid
 * (nz*ny*nx floats); on_device != 0 means device pointers. */
int gpi_set_medium(gpi_plan *plan, const float *const *mod, int on_device);

/* update_pml! result (src/fdtd/cpml.jl:8-155): for derivative field q
 * (canonical order of the physics, see docs) the arrays a, b, kI, each of
 * length len, which must equal 2*npml of the plan (the first npml values
 * serve the min face, the last npml the max face, cpml.jl:88-99). */
int gpi_set_pml(gpi_plan *plan, int q, int len, const float *a, const float *b, const float *kI);

/* Source spray matrix and wavelets of one supersource (fill_wavelets!,
 * src/fdtd/source.jl:24-58, and ssprayw, src/fdtd/ageom.jl:33-45).
 * ipw = 1 for the first wavefield.  ipw = 2 sets the adjoint sources of
 * the second wavefield, injected through the receiver interpolation
 * matrix of `field` (src/fdtd/source.jl:141-156); colptr/rowval/nzval are
 * then ignored and ns must equal the receiver count.  wavelets: nt x ns. */
int gpi_set_sources(gpi_plan *plan, int ipw, int shot, int field, int ns, const int64_t *colptr,
                    const int64_t *rowval, const float *nzval, const float *wavelets);
/* gradient!'s adjoint sources for L2DistLoss (src/fdtd/func_grad.jl:11-49)
 * computed on the device from the records of the last forward_save run of
 * one shot and (velocity) receiver field: the adjoint wavefield's sources of
 * that field become deriv(L2DistLoss(), dobs, dcal) = 2 (dobs - dcal),
 * reversed in time (reverse!(srcwav[2])), injected through the receiver
 * interpolation (as gpi_set_sources(plan, 2, ...) with those wavelets);
 * *misfit = sum (dobs - dcal)^2 in double (value(L2DistLoss(), dobs, dcal)).
 * dobs: nt x nr (Recs layout), host or device (on_device).  Synchronises
 * the plan's stream (the misfit is read back). */
int gpi_set_adjoint_l2(gpi_plan *plan, int shot, int field, const float *dobs, int on_device, double *misfit);
/* Remove every source of wavefield ipw of one shot (-1: all shots). */
int gpi_clear_sources(gpi_plan *plan, int ipw, int shot);
/* Receiver interpolation matrix (rinterpolatew, src/fdtd/ageom.jl:46-54). */
int gpi_set_receivers(gpi_plan *plan, int shot, int field, int nr, const int64_t *colptr,
                      const int64_t *rowval, const float *nzval);

/* Born modelling (FdtdAcoustic{Born}, update!(pa, medium, medium_pert),
 * src/fdtd/medium.jl:103-126; the reference's secondary-source kernels,
 * src/fdtd/born.jl:1-13, pass arguments its kernels do not take, so the
 * engine implements the exact linearisation of its own scheme instead).
 * dmod[0], dmod[1]: the perturbations of invK and rho on the extended grid
 * (nz*nx floats each; on_device != 0 for device pointers).  A later
 * gpi_run(plan, GPI_BORN) propagates wavefield 1 (the background, with the
 * plan's sources) and wavefield 2, which has no sources of its own: after
 * wavefield 1's velocity update each velocity cell of wavefield 2 gains
 * rv (v1 - v1_prev), with rv = -(drho_a + drho_b) / (rho_a + rho_b) over
 * the two density cells of the cell's update coefficient, and after the
 * pressure update each p cell gains -(dinvK / invK) (p1 - p1_prev).
 * gpi_get_records then returns wavefield 2's records (the Born data).
 * 2-D acoustic plans with npw = 2 only. */
int gpi_set_born(gpi_plan *plan, const float *const *dmod, int on_device);

/* mod_x_proc! over every shot of the plan in the given mode
 * (src/fdtd/propagate.jl:74-261).  Asynchronous on the plan's stream. */
int gpi_run(gpi_plan *plan, int mode);

/* update_datamat!/update_data! (src/fdtd/receiver.jl:17-46): records of
 * one shot and field as nt x nr (column-major, Recs.d layout). */
int gpi_get_records(gpi_plan *plan, int shot, int field, float *out, int on_device);
/* sum_grads! (src/fdtd/gradient.jl:2-14): the gradient w.r.t. medium
 * parameter `param`, summed over the plan's shots, on the extended grid. */
int gpi_get_gradient(gpi_plan *plan, int param, float *out, int on_device);
/* Final state of a field of wavefield ipw for one shot (w1[:t]) in its
 * reference shape. */
int gpi_get_field(gpi_plan *plan, int ipw, int shot, int field, float *out, int on_device);
/* Snapshots (tsnaps / snaps_field of PFdtd, src/fdtd/fdtd.jl:179-187;
 * snaps_save!, src/fdtd/fdtd.jl:586-591, called at the end of step it,
 * src/fdtd/propagate.jl:238-245): every later run keeps, after step its[k]
 * (1-based) of the time loop, the field `field` of each active wavefield on
 * the device.  field < 0 or n = 0 turns them off.  A checkpointed adjoint
 * run takes none. */
int gpi_set_snapshots(gpi_plan *plan, int field, int n, const int *its);
/* Snapshot k (order of `its`) of wavefield ipw (1 or 2) for one shot, in
 * the field's reference shape (pa[:snaps, iss]). */
int gpi_get_snapshot(gpi_plan *plan, int ipw, int k, int shot, float *out, int on_device);
/* Source illumination (illum_flag of PFdtd, src/fdtd/fdtd.jl:59,73,177;
 * compute_illum!, src/fdtd/fdtd.jl:571-582, at the end of every step of the
 * loop, src/fdtd/propagate.jl:236; stack_illums!, src/fdtd/fdtd.jl:556-566).
 * enable != 0: every later run sums, per shot and cell, p^2 of wavefield 1
 * over its steps (the square in FP32, the sum in FP64); acoustic media only
 * (GPI_E_UNSUPPORTED otherwise).  A checkpointed adjoint run keeps the sums
 * of its forward_save run.  The reference declares the flag and both
 * functions but leaves their calls commented out (its illum_stack stays 0). */
int gpi_set_illum(gpi_plan *plan, int enable);
/* The illumination of the last run summed over shots (shot order, from 0)
 * on the physical grid (the padded PML cells dropped): FP64, column-major,
 * z fastest, nz_phys x [ny_phys x] nx_phys values. */
int gpi_get_illum(gpi_plan *plan, double *out, int on_device);
/* Number of engine kernel launches issued by the last gpi_run. */
int gpi_last_launches(const gpi_plan *plan, int64_t *launches);

/* CUDA graphs for later gpi_run calls of this plan.  enable = 1: each run
 * as one graph per mode, captured on its first run (after the sources and
 * receivers are compiled) and replayed, which removes the per-launch host
 * cost of small grids for plans that run repeatedly.  enable = 2: each run
 * as replays of one captured chunk of 16 steps that reads the step from a
 * device counter, so that a plan that runs once gains too (the checkpointed
 * forward_save and adjoint runs stay plain).  0: plain launches.  Changing the sources or receivers
 * drops the graphs.  No counterpart in the reference (its time loop
 * launches every kernel). */
int gpi_set_graph(gpi_plan *plan, int enable);
/* Non-blocking completion test of the plan's stream (1 when all work
 * issued so far has finished).  No counterpart in the reference. */
int gpi_query(gpi_plan *plan, int *done);
/* The binomial checkpoint schedule of a checkpointed adjoint over nt steps
 * with `slots` state slots (host only, no device needed): forward steps it
 * recomputes besides its turns, turns (= nt), slots the forward_save run
 * fills.  No counterpart in the reference. */
int gpi_checkpoint_schedule(int nt, int slots, int64_t *advances, int64_t *turns, int *stored);

/* ------------------------------------------------------------------------
 * Serving (no counterpart in the reference, whose update!(pa) runs one
 * experiment at a time on each Distributed worker,
 * src/fdtd/propagate.jl:100-106).  A server admits queued requests in
 * arrival order (within each kind below) while the device bytes of the
 * admitted ones stay within its HBM budget.  Small 2-D forward requests (up
 * to 4 Mi cells per step over their shots) join the batch of their physics
 * (gpi_batch_*): one launch per tile class and time step advances every
 * admitted one, and requests join and leave it as they arrive and finish.
 * Larger forward, gradient and 3-D requests run up to max_inflight at
 * once on their own streams (host set-up of one overlapping the device work
 * of the others; each request's shots batched into every launch, forward
 * runs replayed as captured step chunks).  Results stay on the host until
 * released; a request's results do not depend on what else runs.
 * ------------------------------------------------------------------------ */
typedef struct gpi_server gpi_server;

typedef struct {
  int32_t device;       /* CUDA device of every request */
  int32_t max_inflight; /* gradient and 3-D requests on the device at once
                           (1..64 worker threads) */
  int32_t max_batch;    /* 2-D forward requests advanced together by one batch
                           (gpi_batch_*) per physics (0: 16; -1: none, they run
                           on the worker threads like the others) */
  int32_t reserved;
  size_t hbm_budget;    /* device bytes the admitted requests may hold together
                           (a request larger than the budget runs alone) */
} gpi_server_desc;

/* One sparse projection of one shot and field (as gpi_set_sources /
 * gpi_set_receivers take it) with its time series. */
typedef struct {
  int32_t shot, field, n, pad;
  const int64_t *colptr, *rowval; /* CSC, 0-based */
  const float *nzval;
  const float *data; /* sources: wavelets nt x n (required); receivers of a
                        gradient request: observed records nt x n (NULL:
                        zero); receivers of a forward request: ignored */
} gpi_proj;

typedef struct {
  gpi_plan_desc plan;      /* npw = 1 for a forward request, 2 for a gradient */
  int32_t gradient;        /* 0: update!(pa); 1: gradient!(g, m, L2DistLoss(),
                              dobs, pa) (src/fdtd/func_grad.jl:11-49) */
  int32_t nsrc, nrec;      /* entries of src (wavefield-1 sources) and rec */
  int32_t graph;           /* gpi_set_graph kind for the request's runs */
  const float *const *mod; /* host medium parameters on the extended grid */
  const float *pml;        /* host CPML profiles: per derivative field q
                              (canonical order) a, b, kI of 2*npml each */
  const gpi_proj *src, *rec;
} gpi_request;

int gpi_server_create(const gpi_server_desc *desc, gpi_server **out);
/* Stops admitting, lets running requests finish, frees everything. */
void gpi_server_destroy(gpi_server *server);
/* Copies the request (the caller may free its arrays on return) and queues
 * it; *id identifies it.  Returns at once. */
int gpi_server_submit(gpi_server *server, const gpi_request *req, int64_t *id);
/* *state: 0 queued, 1 running, 2 done, 3 failed. */
int gpi_server_poll(gpi_server *server, int64_t id, int *state);
/* Blocks until the request is done; returns its status. */
int gpi_server_wait(gpi_server *server, int64_t id);
/* Records (nt x n, column-major) of one receiver entry of a done request. */
int gpi_server_records(gpi_server *server, int64_t id, int shot, int field, float *out);
/* Raw gradient accumulations summed over shots (param as gpi_get_gradient,
 * extended grid; out may be NULL) and the misfit of a gradient request. */
int gpi_server_gradient(gpi_server *server, int64_t id, int param, float *out, double *loss);
/* t[0..2]: submission, admission and completion times in seconds since the
 * server was created. */
int gpi_server_times(gpi_server *server, int64_t id, double *t);
/* Message of a failed request (or, for an unknown id, of the last failing
 * server call on this thread). */
const char *gpi_server_message(gpi_server *server, int64_t id);
/* Frees a done or failed request's results. */
int gpi_server_release(gpi_server *server, int64_t id);

/* ---- batches: several forward plans advanced by the same launches ----
 * No counterpart in the reference (its update!(pa) runs one experiment at a
 * time per Distributed worker, src/fdtd/propagate.jl:100-106); the serving
 * loop uses it for 2-D forward requests.  Every time step of a batch issues
 * the source / record work of every member and one launch per tile class of
 * the step kernel over the tiles of all members (runs of 16 steps replayed as
 * a captured graph); a member's results equal its own gpi_run(plan,
 * GPI_FORWARD) bit for bit. */
typedef struct gpi_batch gpi_batch;
/* stream: cudaStream_t the batch runs on (NULL: its own). */
int gpi_batch_create(int device, void *stream, gpi_batch **out);
/* A prepared 2-D forward plan (npw = 1, no snapshots, not Born; the same
 * physics as the batch's other members) starts its run at step 1; its set-up
 * work on its own stream is ordered before its first step.  The plan then
 * belongs to the batch until it is handed back by gpi_batch_finished. */
int gpi_batch_add(gpi_batch *batch, gpi_plan *plan);
/* Issues up to max_steps steps of every member, asynchronously on the
 * batch's stream; a member that reaches its last step runs the rest of its
 * run (the last velocity records, the extra velocity half step) and leaves
 * the batch.  *active: the members left (may be NULL). */
int gpi_batch_advance(gpi_batch *batch, int max_steps, int *active);
/* The plans whose runs were issued to the end since the last call (up to
 * cap, oldest first), handed back: later calls on such a plan (records,
 * destroy) wait for its own work only. */
int gpi_batch_finished(gpi_batch *batch, gpi_plan **plans, int cap, int *n);
int gpi_batch_launches(gpi_batch *batch, int64_t *n);
const char *gpi_batch_error(const gpi_batch *batch);
/* Waits for the batch's work; members still in it keep their state. */
void gpi_batch_destroy(gpi_batch *batch);

/* Size of the device scratch array used by gpi_forward_acoustic2d_noalloc. */
#define GPI_NOALLOC_SCRATCH_BYTES (64u << 20)

/* A complete 2-D acoustic forward run (one shot, order 4) that allocates no
 * device memory.  No counterpart in the reference: it is for hosts that
 * cannot call cudaMalloc while they model -- a process whose HBM budget is
 * reserved up front by its own pool allocator, or a latency-critical loop
 * that must not hit cudaMalloc/cudaFree, which can synchronise the device.
 * All intermediates live in one static device array of
 * GPI_NOALLOC_SCRATCH_BYTES per GPU (held until the process exits); larger
 * problems are rejected with GPI_E_INVALID.  Calls share that array: calls
 * that overlap on the GPU race.  The first call on a device looks up the
 * array's address with that device current and keeps it until the process
 * exits; make it before any stream capture begins, and do not reset the
 * device while the library is loaded.
 *   desc      physics GPI_ACOUSTIC, ndim 2, order 4, nshots 1, npw 1
 *   invK, rho device, extended grid, column-major (nz*nx each)
 *   pml       device, 4 x 3 x 2*npml floats: a, b, kI of dpdx, dpdz, dvxdx, dvzdz
 *   src_*     one spray matrix (host CSC, as gpi_set_sources) on src_field
 *             (GPI_P, GPI_VX or GPI_VZ); wavelets: device, nt x ns
 *   rfields   nrf (<= 3) receiver fields among p, vx, vz, each with nr[k]
 *             (<= 4096) receivers as host CSC; records[k]: device, nt x nr[k]
 * Runs on `stream` (cudaStream_t) and synchronises it before returning
 * (once after the table uploads, once to read the kernels' error flag), so
 * the host blocks until the records are written.  GPI_E_CUDA if a CUDA
 * call failed or a kernel's bounded pipeline wait gave up. */
int gpi_forward_acoustic2d_noalloc(const gpi_plan_desc *desc, const float *invK, const float *rho, const float *pml,
                                   int src_field, int ns, const int64_t *src_colptr, const int64_t *src_rowval,
                                   const float *src_nzval, const float *wavelets, int nrf, const int *rfields,
                                   const int *nr, const int64_t *const *rec_colptr, const int64_t *const *rec_rowval,
                                   const float *const *rec_nzval, float *const *records, void *stream);

#ifdef __cplusplus
}
#endif
#endif
