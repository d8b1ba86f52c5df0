// gpi_internal.cuh -- device layout and plan state of the GB300 FDTD engine.
//
// Storage layout (one array per field, per buffer, per wavefield):
//   every field of a shot lives in an NZP x [NYP x] NXP block, z fastest,
//   with a front pad of ZOFF rows / YOFF planes / XOFF columns, so that the
//   reference's 1-based index (r, [y,] c) of ANY field sits at
//       off = ((c - 1 + XOFF) * NYP + (y - 1 + YOFF)) * NZP + (r - 1 + ZOFF)
//   (NYP = 1, YOFF = 1 in 2-D).  Fields of different staggered shapes thus
//   share one index map and the pads absorb the stencil halos, so kernels
//   need no bounds checks on reads.  NZP is a multiple of 32 floats, so a
//   column starts on a 128-byte boundary.  Shots are stacked behind each
//   other (shot stride = NZP * NYP * NXP).
//
//   State is double-buffered (ping-pong): a time step reads buffer `cur`
//   and writes buffer `cur ^ 1`, which lets one kernel advance velocities
//   and stresses together while neighbouring blocks recompute halo
//   velocities from untouched inputs.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gpi_fdtd.h"

namespace gpi {

constexpr int NFIELD = 10;
constexpr int ZOFF = 4, XOFF = 4, YOFF = 4;
constexpr int MAXDER = 18;
constexpr int NKIND = 4;  // injection kinds: vx, vy, vz, stress
// rows of a 2-D step-kernel block: 124 stress rows + 3 halo velocity rows
// fill four warps; a multiple of 4 keeps every column copy 16-byte aligned
constexpr int TZ2 = 124;

// Canonical derivative order (docs and oracle use the same):
//   A2: dpdx dpdz dvxdx dvzdz
//   E2: dtauxxdx dtauxzdx dtauzzdz dtauxzdz dvxdx dvzdz dvxdz dvzdx
//   A3: dpdx dpdy dpdz dvxdx dvydy dvzdz
//   E3: dtauxxdx dtauxydx dtauxzdx dtauyydy dtauxydy dtauyzdy dtauzzdz
//       dtauyzdz dtauxzdz dvxdx dvydy dvzdz dvxdy dvxdz dvydx dvydz dvzdx dvzdy
struct DerivSpec {
  int axis;        // 0 z, 1 y, 2 x
  int kz, ky, kx;  // shape kinds: 0 n, 1 n+h, 2 n-h, 3 n-2h
};
int deriv_specs(int physics, int ndim, const DerivSpec **out);
void field_kinds(int field, int *kz, int *ky, int *kx);

// One receiver (one CSC column) of one (shot, field).
struct RecTask {
  int32_t shot, field, e0, e1;  // entries [e0, e1)
  int64_t out;                  // offset of record (it=0) in the record pool
  int32_t stride;               // floats between consecutive time samples
  int32_t pad;
};
// One injection cell (one row of one spray matrix) of one (shot, ipw, kind).
struct InjCell {
  int32_t row, col, ydx;  // reference 1-based indices in the target field (ydx = y in 3-D)
  int32_t kind;           // 0 vx, 1 vy, 2 vz, 3 stress (p or the normal stresses)
  int32_t e0, e1;         // (source, weight) pairs [e0, e1)
  int32_t wav;            // index of the wavelet table entry (ns, pointer)
  int32_t pad;
  int64_t off;            // storage offset within the shot
  int64_t roff0, roff1;   // rho storage offsets of the density average (velocity kinds)
};

struct Plan {
  gpi_plan_desc d;
  int h = 3;
  int NZP = 0, NYP = 1, NXP = 0;
  int64_t fstride = 0;  // floats per field per shot
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int present[NFIELD] = {0};
  int nder = 0;
  const DerivSpec *ds = nullptr;
  // tiling of the step kernel
  int TZ = 128, TY = 1, L = 128, nzb = 1, nyb = 1, nxb = 1;
  std::vector<int> xcut;  // 2-D: x-chunk b covers columns [xcut[b], xcut[b + 1])

  // device memory
  void *pool = nullptr;
  size_t pool_bytes = 0;
  float *state[2][2][NFIELD] = {};  // [buffer][ipw][field] -> shot 0
  float *psi[2][2][MAXDER] = {};    // [buffer][ipw][q]
  int64_t psi_stride[MAXDER] = {};  // floats per shot
  float *coef[8] = {};              // update coefficients, storage layout
  int ncoef = 0;
  float *mod[3] = {};  // medium parameters, storage layout
  int nmod = 0;
  float *pml = nullptr;  // [nder][3][2*npml]
  float *grad[3] = {};   // per-shot gradients [shot][storage] (adjoint), one per medium parameter
  // stencil orders other than 4 (k_generic.cu): 1 / (den * d) per axis (z, y, x)
  float gdsI[3] = {0.f, 0.f, 0.f};
  // 2-D acoustic adjoint by time reversal: per velocity cell and shot, the
  // sums over the steps of vx2_prev (vx1 - vx1_prev) / dt (img[0]) and of
  // the vz products (img[1]); the rho gradient is formed from them at the
  // end of the run
  float *img[2] = {};
  float *bstore = nullptr;  // boundary store (forward_save -> adjoint)
  float *bprev = nullptr;   // adjoint: the strip values the forcing replaced, this step
  int64_t bstep = 0;         // floats per step per shot
  int64_t bsnap = 0;         // floats of the final snapshots per shot
  int cur[2] = {0, 0};       // buffer holding the current state, per wavefield
  int have_save = 0;

  // receivers
  std::vector<std::vector<int>> rec_n;               // [shot][field] -> nr (0 none)
  std::vector<std::vector<std::vector<int64_t>>> rec_cp;   // host copies
  std::vector<std::vector<std::vector<int64_t>>> rec_off;  // storage offsets
  std::vector<std::vector<std::vector<float>>> rec_w;
  float *rec_pool = nullptr;
  size_t rec_pool_floats = 0;
  std::vector<std::vector<int64_t>> rec_base;  // [shot][field] offset in pool
  RecTask *d_rtask = nullptr;
  int n_rtask = 0;
  int64_t *d_roff = nullptr;
  float *d_rw = nullptr;
  bool rec_dirty = true;

  // sources: per (ipw, shot, field) CSC + wavelets (host), compiled to cells
  struct Src {
    int ns = 0;
    std::vector<int64_t> cp, rv;
    std::vector<float> nz, wav;
    bool on_dev = false;  // the adjoint wavefield's wavelets are in adj_dev (gpi_set_adjoint_l2)
  };
  std::vector<std::vector<std::vector<Src>>> src;  // [ipw][shot][field]
  std::vector<std::vector<float *>> adj_dev;       // [shot][field]: device wavelets of the adjoint sources
  bool src_dirty = true;
  InjCell *d_cells = nullptr;
  int n_cells = 0;
  int32_t *d_pair_j = nullptr;
  float *d_pair_w = nullptr;
  float **d_wav = nullptr;  // per wavelet table entry: device pointer (nt x ns)
  int32_t *d_wav_ns = nullptr;
  std::vector<float *> wav_bufs;
  float *d_amount = nullptr;               // per cell, current step
  std::vector<int32_t> group_ptr;          // [(ipw*nshots + shot)*NKIND + kind] -> cell range
  bool inj_shared = false;                 // some group holds one storage cell twice
  int32_t *d_group_ptr = nullptr;

  int64_t launches = 0;
  int *d_err = nullptr;  // set by a kernel whose pipeline wait gave up
  // tiles of the 2-D step kernels (z-block, first column, end column, shot),
  // grouped by class: interior, band, x-band, edge (classify_tiles)
  int4 *d_tiles = nullptr;
  int n_tiles[4] = {0, 0, 0, 0};
  // the most injection cells (columns x0 .. x1+2 of a tile, every kind) a
  // tile of each class holds: wavefield 1, wavefield 2, both; sizes the
  // shared-memory copy of the 2-D acoustic step kernel (0: none)
  int inj_tile[3][4] = {};
  std::vector<int4> h_tiles;  // host copy of the tile list (batches tag and concatenate them)
  // 2-D z-strip CPML memory: column stride and the window of a column that
  // the general step kernel stages per ring slot
  int zsw = 0, pzw = 0;
  // side streams for the edge, x-band and band step kernels, so that their
  // blocks and the interior kernel's share the SMs (fork and join events on
  // the plan stream)
  static constexpr int NSIDE = 3;
  cudaStream_t side[NSIDE] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[NSIDE] = {};
  // CUDA graphs (gpi_set_graph): 1 the whole run per mode, 2 forward runs
  // as replays of one captured chunk of kChunkSteps steps that read the
  // step from d_it
  bool use_graph = false;
  int graph_kind = 0;
  cudaStream_t own_stream = nullptr;  // created for graphs when no stream was given
  cudaGraphExec_t gexec[3] = {};
  int64_t glaunches[3] = {};
  cudaGraphExec_t cexec[3] = {};
  int64_t claunches[3] = {};
  int *d_it = nullptr;
  std::vector<InjCell> h_cells;  // host copy of the injection cells (tile classification)

  // Born modelling (gpi_set_born): secondary-source ratios of p, vx, vz in
  // the storage layout of one shot (zero outside the update domains), and
  // the uploaded perturbations
  float *born = nullptr;  // [5][fstride]: rp, rvx, rvz, dinvK, drho
  bool have_born = false;
  int rec_ipw = 0;  // wavefield the records are gathered from (1: Born runs)

  // snapshots (gpi_set_snapshots): field, steps, device copies
  // [ipw][k][shot][storage]
  int snap_field = -1;
  std::vector<int> snap_its;
  float *snap_buf = nullptr;

  // source illumination (gpi_set_illum): per shot, sum over the steps of a
  // run of p^2 of wavefield 1, FP64, storage layout [shot][storage]
  double *illum = nullptr;

  // checkpointed adjoint (gpi_plan_desc.checkpoints > 0): full states of
  // wavefield 1 (fields and CPML memory) in ck_slots device slots instead of
  // the boundary store; the adjoint run recomputes forward states from them
  // on a binomial schedule
  int ck_slots = 0;
  float *ck_pool = nullptr;
  int64_t ck_floats = 0;                     // floats per slot
  std::vector<std::pair<int, int>> ck_first;  // (state, slot) the forward_save run stores
  std::vector<std::vector<Src>> ck_src;      // wavefield-1 sources of the forward_save run
};

// error helpers
int fail(Plan *p, int code, const std::string &msg);
#define GPI_CUDA(p, call)                                                              \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) return gpi::fail((p), GPI_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

inline int64_t soff(const Plan &p, int r, int y, int c) {
  return ((int64_t)(c - 1 + XOFF) * p.NYP + (p.d.ndim == 3 ? (y - 1 + YOFF) : 0)) * p.NZP + (r - 1 + ZOFF);
}
int nkind(int kind, int n, int h);

// 2-D CPML memory of a z strip is stored as one column of 2*npml slots (top
// strip, then bottom strip) per x index; the column stride is padded to 16
// bytes so that a column window moves with one bulk copy.
__host__ __device__ inline int zstrip_stride(int npml) { return (2 * npml + 3) & ~3; }
// z strips read by a block of TZ rows starting at z0 (velocity halo and
// mirror rows included, with margin): bit 0 the top strip, bit 1 the bottom
__host__ __device__ inline int zstrip_touch(int z0, int TZ, int nz, int npml, bool lo, bool hi) {
  int m = 0;
  if (lo && z0 - 8 <= npml) m |= 1;
  if (hi && z0 + TZ + 8 > nz - 6 - npml) m |= 2;
  return m;
}
// first strip slot of the staged window of pzw slots (pzw from zstrip_window)
__host__ __device__ inline int zstrip_off(int touch, int zsw, int pzw) { return touch == 2 ? zsw - pzw : 0; }
// slots per column a block stages: the top half (from slot 0), the bottom
// half (ending at the padded stride) or the whole column when a block meets
// both strips; the largest over the z blocks of the plan
inline int zstrip_window(int nzb, int TZ, int nz, int npml, bool lo, bool hi) {
  const int zsw = zstrip_stride(npml);
  int w = 0;
  for (int zb = 0; zb < nzb; zb++) {
    const int m = zstrip_touch(1 + zb * TZ, TZ, nz, npml, lo, hi);
    const int need = m == 3 ? zsw : m == 1 ? (npml + 3) / 4 * 4 : m == 2 ? zsw - (npml & ~3) : 0;
    w = w > need ? w : need;
  }
  return w;
}

// kernels (per physics)
int step_acoustic2d(Plan *p, int ipw_mask, int it, int mode, int vonly);
int step_elastic2d(Plan *p, int ipw_mask, int it, int mode, int vonly);
int step_acoustic3d(Plan *p, int ipw_mask, int it, int mode, int vonly);
int step_elastic3d(Plan *p, int ipw_mask, int it, int mode, int vonly);
int step_adjoint_acoustic2d(Plan *p, int it);
int step_a2_wavefield(Plan *p, int ipw, int vonly);
int step_a2_adjoint_fused(Plan *p);  // both wavefields + imaging condition
int step_generic(Plan *p, int vonly);  // stencil orders 2, 6, 8 (k_generic.cu)
// source illumination (k_common.cu): add p^2 of wavefield 1 to the per-shot
// sums; the shot stack over the cells of the physical grid
int illum_add(Plan *p);
int illum_stack(Plan *p, double *dst);
// batches of forward plans (gpi_batch.cu): argument tables and launches of
// the step kernels over the tagged tiles of several plans
size_t a2_args_bytes();
void a2_batch_args(Plan *p, void *out, size_t smem[4]);
int a2_batch_launch(Plan *p, int m, const void *args, const int4 *tiles, int n, int par, size_t smem, cudaStream_t st);
size_t e2_args_bytes();
void e2_batch_args(Plan *p, void *out, size_t smem[4]);
int e2_batch_launch(Plan *p, int m, const void *args, const int4 *tiles, int n, int par, size_t smem, cudaStream_t st);
int adjoint_l2_launch(Plan *p, float *adj, double *partial, double *out, const float *dobs, const float *rec, int nt,
                      int nr);
int adjoint_l2_blocks(int nt, int nr);
size_t aux_args_bytes();
int aux_batch_args(Plan *p, void *out);  // returns its block count
int aux_batch_launch(Plan *p, const void *args, const int *first, int nplans, int nblocks, int par, int off,
                     cudaStream_t st);
int run_prepare_forward(Plan &p);
cudaError_t pool_alloc(void **ptr, size_t bytes, cudaStream_t st);  // the engine's memory pool
int run_finish_forward(Plan &p);
int img_rho_finish(Plan *p);         // the rho gradient from img[0], img[1]
int step3_wavefield(Plan *p, int ipw, int vonly);
// checkpointed adjoint (gpi_ckpt.cu)
int64_t ckpt_slot_floats(const Plan &p);
int ckpt_forward_store(Plan *p, int it);  // after forward_save step it
int ckpt_adjoint(Plan *p);                 // the whole adjoint run
int aux_step2(Plan *p, int it1, int it2);
// raise a kernel's dynamic shared-memory limit on the current device to
// `bytes` once (thread-safe: plans on several host threads share it)
int ensure_smem_attr(Plan *p, const void *fn, int slot, size_t bytes);
int aux_step_dev(Plan *p, int off, int mode);  // step *d_it + off
int set_step(Plan *p, int v, int add);         // *d_it = v, or += v
constexpr int kChunkSteps = 16;                // steps per replayed chunk (even: ping-pong)
// host: x partition of a 2-D grid of nx columns into m interior chunks
// plus, when the grid is wide enough, one narrow chunk at each x edge (the
// mirror columns there need the general code) and one chunk over each x
// CPML strip (split to the interior chunk width); writes nchunks + 1 cut
// columns (at most m + 2 npml + 8), returns nchunks
int make_xcuts(int nx, int m, int npml, bool xlo, bool xhi, int *cuts);
// host: classify the (z-block, x-chunk, shot) tiles of a 2-D plan and write
// them grouped by class (0 interior, 1 band, 2 x-band, 3 edge, in that
// order) with the per-class counts; returns the tile count (or -1 beyond
// `cap`)
int classify_tiles(const Plan &p, const int *xcut, const InjCell *cells, const int32_t *gptr, int4 *out, int cap,
                   int count[4]);
int aux_step(Plan *p, int it, int mode);
void drop_graphs(Plan &p);
// nside side streams forked from the plan stream (the plan stream itself
// when side streams are unavailable); join_side joins them back
int fork_side(Plan *p, int nside, cudaStream_t *out);
int join_side(Plan *p, int nside);
int compute_coefficients(Plan *p);
int boundary_io(Plan *p, int it, int dir);
int boundary_io_dev(Plan *p, int off, int dir);  // step *d_it + off
int snap_io(Plan *p, int tau, int dir);
// Born modelling (k_born.cu)
int born_coefficients(Plan *p);
int born_run(Plan *p);

}  // namespace gpi

struct gpi_plan {
  gpi::Plan p;
};
