// k_noalloc.cu -- a 2-D acoustic forward run that allocates no device memory.
//
// Some hosts cannot call cudaMalloc while they model: a service that has
// reserved its whole HBM budget in its own pool allocator at start-up (and
// must not let a library grow the process's footprint behind the pool's
// back), or a latency-critical loop that must not hit cudaMalloc/cudaFree,
// which can synchronise the whole device and stall every other stream.  For
// them gpi_forward_acoustic2d_noalloc runs the same kernels as the plan
// path (the fused 2-D acoustic step kernel and the per-step auxiliary
// kernel), with every intermediate -- both ping-pong wavefield buffers, the
// CPML memory, the update coefficients, the record buffer and the source /
// receiver tables -- carved out of one file-scope __device__ array of
// GPI_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU that loads the library
// holds that array until the process exits.  The caller passes the medium,
// the PML profiles and the wavelets as device arrays and receives the
// records in device arrays it owns.
//
// The array is shared by every call: each call clears the parts that must
// start at zero, and two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on it.  The first call on a
// device looks up the device address of the array (cudaGetSymbolAddress)
// with that device current and keeps it for the life of the process; make
// that first call before any stream capture begins, and do not reset the
// device (cudaDeviceReset) while the library is loaded.  Every call
// synchronises `stream` twice -- after the table uploads, because the host
// staging tables are static and reused by the next call, and at the end, to
// read the kernels' error flag -- so it returns when the run has finished.
#include <algorithm>
#include <mutex>
#include <string>

#include "gpi_internal.cuh"

namespace gpi {

int transpose_records(Plan *p, float *out, const float *in, int nt, int nr);  // k_common.cu

static constexpr size_t kScratchFloats = (size_t)GPI_NOALLOC_SCRATCH_BYTES / sizeof(float);
static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

static std::mutex g_mu;
static constexpr int kMaxDevices = 64;
static float *g_scratch_addr[kMaxDevices] = {};

// host staging, static so that the call needs no heap (guarded by g_mu)
static constexpr int kMaxRecFields = 3, kMaxRec = 4096, kMaxRecEntries = 4 * kMaxRec * kMaxRecFields;
static constexpr int kMaxCells = 1024, kMaxPairs = 4096;
static RecTask h_tasks[kMaxRec * kMaxRecFields];
static int64_t h_roff[kMaxRecEntries];
static float h_rw[kMaxRecEntries];
static InjCell h_cells[kMaxCells];
static int32_t h_pj[kMaxPairs];
static float h_pw[kMaxPairs];
static int32_t h_gptr[2 * NKIND + 1];
static float *h_wavptr[1];
static constexpr int kMaxTiles = 1 << 16, kMaxCuts = 1 << 13;
static int4 h_tiles[kMaxTiles];
static int h_xcut[kMaxCuts];
static Plan g_plan;  // descriptor filled per call; its pointers point into the scratch

static int h_err;  // the kernels' error flag, read back at the end of a call

static int nfail(int code, const char *msg) { return fail(nullptr, code, msg); }

#define NA_CUDA(call)                                                   \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) return nfail(GPI_E_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// device address of the scratch on the current device (looked up once)
static int scratch_base(float **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nfail(GPI_E_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return nfail(GPI_E_UNSUPPORTED, "device index too large");
  if (!g_scratch_addr[dev]) {
    float *ptr = nullptr;
    e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) return nfail(GPI_E_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return GPI_OK;
}

static int shape_of(const Plan &p, int f, int n[3]) {
  int kz, ky, kx;
  field_kinds(f, &kz, &ky, &kx);
  n[0] = nkind(kz, p.d.nz, p.h);
  n[1] = 1;
  n[2] = nkind(kx, p.d.nx, p.h);
  return n[0] * n[2];
}

}  // namespace gpi

using namespace gpi;

extern "C" int gpi_forward_acoustic2d_noalloc(const gpi_plan_desc *desc, const float *invK, const float *rho,
                                              const float *pml, int src_field, int ns, const int64_t *src_colptr,
                                              const int64_t *src_rowval, const float *src_nzval,
                                              const float *wavelets, int nrf, const int *rfields, const int *nr,
                                              const int64_t *const *rec_colptr, const int64_t *const *rec_rowval,
                                              const float *const *rec_nzval, float *const *records, void *stream) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!desc || !invK || !rho || !pml || !wavelets) return nfail(GPI_E_INVALID, "null argument");
  const gpi_plan_desc &d = *desc;
  if (d.physics != GPI_ACOUSTIC || d.ndim != 2 || d.order != 4 || d.nshots != 1 || d.npw != 1)
    return nfail(GPI_E_UNSUPPORTED, "no-alloc path: 2-D acoustic, order 4, one shot, one wavefield");
  if (d.nt < 1 || d.npml < 1 || !(d.dt > 0) || !(d.dz > 0) || !(d.dx > 0)) return nfail(GPI_E_INVALID, "descriptor");
  if (std::min(d.nz, d.nx) - 6 < 2 * d.npml + 1) return nfail(GPI_E_INVALID, "grid too small for two PML strips");
  if (src_field != GPI_P && src_field != GPI_VX && src_field != GPI_VZ) return nfail(GPI_E_INVALID, "source field");
  if (ns < 1 || !src_colptr || !src_rowval || !src_nzval) return nfail(GPI_E_INVALID, "source matrix");
  if (nrf < 0 || nrf > kMaxRecFields) return nfail(GPI_E_INVALID, "at most 3 receiver fields");
  if (nrf > 0 && (!rfields || !nr || !rec_colptr || !rec_rowval || !rec_nzval || !records))
    return nfail(GPI_E_INVALID, "null receiver array");
  float *base = nullptr;
  int rc = scratch_base(&base);
  if (rc) return rc;

  // ---- layout (same storage map as a plan) ----
  Plan &P = g_plan;
  P.d = d;
  P.d.ny = 1;
  P.d.rigid_faces |= d.pml_faces;
  P.h = 3;
  P.stream = (cudaStream_t)stream;
  P.TZ = TZ2;
  P.nzb = (d.nz + TZ2 - 1) / TZ2;
  P.L = 128;
  {
    const int m = std::max(1, (d.nx - 16 + P.L - 1) / P.L);
    if (m + 2 * d.npml + 8 > kMaxCuts) return nfail(GPI_E_INVALID, "grid too large for the no-alloc tile table");
    P.nxb = make_xcuts(d.nx, m, d.npml, d.pml_faces & GPI_XMIN, d.pml_faces & GPI_XMAX, h_xcut);
  }
  P.nyb = 1;
  P.NZP = (int)(((int64_t)P.nzb * TZ2 + 2 * ZOFF + 4 + 31) / 32 * 32);
  P.NXP = d.nx + 3 + 2 * XOFF + 4;
  P.NYP = 1;
  P.fstride = (int64_t)P.NZP * P.NXP;
  P.zsw = zstrip_stride(d.npml);
  P.pzw = zstrip_window(P.nzb, P.TZ, d.nz, d.npml, d.pml_faces & GPI_ZMIN, d.pml_faces & GPI_ZMAX);
  P.nder = deriv_specs(GPI_ACOUSTIC, 2, &P.ds);
  P.nmod = 2;
  P.ncoef = 3;
  P.pml = (float *)pml;
  P.cur[0] = P.cur[1] = 0;
  P.launches = 0;
  for (int f = 0; f < NFIELD; f++) P.present[f] = f == GPI_P || f == GPI_VX || f == GPI_VZ;
  int64_t used = 0;
  bool room = true;
  auto carve = [&](int64_t nfloat) -> float * {
    float *p = base + used;
    used += (nfloat + 63) / 64 * 64;
    if ((size_t)used > kScratchFloats) room = false;
    return p;
  };
  for (int b = 0; b < 2; b++)
    for (int f : {GPI_P, GPI_VX, GPI_VZ}) P.state[b][0][f] = carve(P.fstride);
  for (int q = 0; q < 4; q++) {
    P.psi_stride[q] = P.ds[q].axis == 2 ? 2 * (int64_t)d.npml * P.NZP : (int64_t)P.NXP * P.zsw;
    for (int b = 0; b < 2; b++) P.psi[b][0][q] = carve(P.psi_stride[q]);
  }
  for (int i = 0; i < 2; i++) P.mod[i] = carve(P.fstride);
  for (int i = 0; i < 3; i++) P.coef[i] = carve(P.fstride);
  P.d_err = (int *)carve(64);

  // ---- receivers: tasks and storage offsets ----
  int ntask = 0, nent = 0;
  int64_t pool = 0;
  for (int k = 0; k < nrf; k++) {
    const int f = rfields[k];
    if ((f != GPI_P && f != GPI_VX && f != GPI_VZ) || nr[k] < 1 || nr[k] > kMaxRec || !records[k] || !rec_colptr[k] ||
        !rec_rowval[k] || !rec_nzval[k])
      return nfail(GPI_E_INVALID, "receiver field / count / arrays (at most 4096 receivers per field)");
    int n[3];
    const int64_t len = shape_of(P, f, n);
    for (int j = 0; j < nr[k]; j++) {
      RecTask &t = h_tasks[ntask++];
      t.shot = 0;
      t.field = f;
      t.e0 = nent;
      for (int64_t e = rec_colptr[k][j]; e < rec_colptr[k][j + 1]; e++) {
        const int64_t lin = rec_rowval[k][e];
        if (lin < 0 || lin >= len || nent >= kMaxRecEntries) return nfail(GPI_E_INVALID, "receiver entries");
        h_roff[nent] = soff(P, (int)(lin % n[0]) + 1, 1, (int)(lin / n[0]) + 1);
        h_rw[nent++] = rec_nzval[k][e];
      }
      t.e1 = nent;
      t.out = pool + j;
      t.stride = nr[k];
      t.pad = 0;
    }
    pool += (int64_t)nr[k] * d.nt;
  }
  P.n_rtask = ntask;
  P.rec_pool = carve(pool);
  P.rec_pool_floats = (size_t)pool;
  P.d_rtask = (RecTask *)carve((int64_t)(sizeof(RecTask) * ntask + 3) / 4);
  P.d_roff = (int64_t *)carve((int64_t)(sizeof(int64_t) * nent + 3) / 4);
  P.d_rw = carve(nent);

  // ---- source cells (one spray matrix), grouped as the plan path does ----
  {
    int n[3];
    const int64_t len = shape_of(P, src_field, n);
    const int kind = src_field == GPI_VX ? 0 : src_field == GPI_VZ ? 2 : 3;
    int ncell = 0, npair = 0;
    for (int j = 0; j < ns; j++)
      for (int64_t e = src_colptr[j]; e < src_colptr[j + 1]; e++) {
        const int64_t lin = src_rowval[e];
        if (lin < 0 || lin >= len) return nfail(GPI_E_INVALID, "source row outside the field");
        const int r = (int)(lin % n[0]) + 1, c = (int)(lin / n[0]) + 1;
        int at = -1;
        for (int q = 0; q < ncell; q++)
          if (h_cells[q].row == r && h_cells[q].col == c) at = q;
        if (at < 0) {
          if (ncell >= kMaxCells) return nfail(GPI_E_INVALID, "too many source cells (1024)");
          InjCell &cl = h_cells[ncell];
          cl.row = r;
          cl.col = c;
          cl.ydx = 1;
          cl.kind = kind;
          cl.e0 = cl.e1 = 0;
          cl.wav = 0;
          cl.pad = 0;  // number of pairs, until they are laid out below
          cl.off = soff(P, r, 1, c);
          cl.roff0 = cl.roff1 = 0;
          at = ncell++;
        }
        (void)at;
        npair++;
      }
    if (npair > kMaxPairs) return nfail(GPI_E_INVALID, "too many source entries (4096)");
    // pairs per cell in ascending source order; drop velocity cells outside @inn
    int m = 0, np = 0;
    for (int q = 0; q < ncell; q++) {
      InjCell cl = h_cells[q];
      if (kind < 3) {
        const bool in = cl.row - 3 >= 1 && cl.row - 3 <= n[0] - 6 && cl.col - 3 >= 1 && cl.col - 3 <= n[2] - 6;
        if (!in) continue;
        const int z = cl.row - 3, x = cl.col - 3;
        const int zz = z + (kind != 2 ? 3 : 0), xx = x + (kind != 0 ? 3 : 0);
        cl.roff0 = soff(P, zz, 1, xx);
        cl.roff1 = soff(P, zz + (kind == 2), 1, xx + (kind == 0));
      }
      cl.e0 = np;
      for (int j = 0; j < ns; j++)
        for (int64_t e = src_colptr[j]; e < src_colptr[j + 1]; e++) {
          const int64_t lin = src_rowval[e];
          if ((int)(lin % n[0]) + 1 == cl.row && (int)(lin / n[0]) + 1 == cl.col) {
            h_pj[np] = j;
            h_pw[np++] = src_nzval[e];
          }
        }
      cl.e1 = np;
      h_cells[m++] = cl;
    }
    // sort by (column, row): insertion sort keeps equal keys in order
    for (int i = 1; i < m; i++) {
      InjCell x = h_cells[i];
      int k = i - 1;
      while (k >= 0 && (h_cells[k].col > x.col || (h_cells[k].col == x.col && h_cells[k].row > x.row))) {
        h_cells[k + 1] = h_cells[k];
        k--;
      }
      h_cells[k + 1] = x;
    }
    for (int g = 0; g <= 2 * NKIND; g++) h_gptr[g] = g <= kind ? 0 : m;
    P.n_cells = m;
    P.d_cells = (InjCell *)carve((int64_t)(sizeof(InjCell) * (m + 1) + 3) / 4);
    P.d_pair_j = (int32_t *)carve(np + 1);
    P.d_pair_w = carve(np + 1);
    P.d_amount = carve(m + 1);
    P.d_group_ptr = (int32_t *)carve(2 * NKIND + 1);
    P.d_wav = (float **)carve(2);
    h_wavptr[0] = (float *)wavelets;
    const int ntile = classify_tiles(P, h_xcut, h_cells, h_gptr, h_tiles, kMaxTiles, P.n_tiles);
    if (ntile < 0) return nfail(GPI_E_INVALID, "grid too large for the no-alloc tile table");
    P.d_tiles = (int4 *)carve((int64_t)(sizeof(int4) * ntile + 3) / 4);
    if (!room) return nfail(GPI_E_INVALID, "problem exceeds the 64 MiB no-alloc scratch");
    cudaStream_t s = P.stream;
    NA_CUDA(cudaMemcpyAsync(P.d_cells, h_cells, sizeof(InjCell) * m, cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(P.d_pair_j, h_pj, sizeof(int32_t) * np, cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(P.d_pair_w, h_pw, sizeof(float) * np, cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(P.d_group_ptr, h_gptr, sizeof(h_gptr), cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(P.d_wav, h_wavptr, sizeof(h_wavptr), cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(P.d_tiles, h_tiles, sizeof(int4) * ntile, cudaMemcpyHostToDevice, s));
  }
  if (!room) return nfail(GPI_E_INVALID, "problem exceeds the 64 MiB no-alloc scratch");
  cudaStream_t s = P.stream;
  NA_CUDA(cudaMemcpyAsync(P.d_rtask, h_tasks, sizeof(RecTask) * ntask, cudaMemcpyHostToDevice, s));
  NA_CUDA(cudaMemcpyAsync(P.d_roff, h_roff, sizeof(int64_t) * nent, cudaMemcpyHostToDevice, s));
  NA_CUDA(cudaMemcpyAsync(P.d_rw, h_rw, sizeof(float) * nent, cudaMemcpyHostToDevice, s));
  // the wavefields, CPML memory and records start at zero
  for (int b = 0; b < 2; b++) {
    for (int f : {GPI_P, GPI_VX, GPI_VZ}) NA_CUDA(cudaMemsetAsync(P.state[b][0][f], 0, P.fstride * sizeof(float), s));
    for (int q = 0; q < 4; q++) NA_CUDA(cudaMemsetAsync(P.psi[b][0][q], 0, P.psi_stride[q] * sizeof(float), s));
  }
  if (pool) NA_CUDA(cudaMemsetAsync(P.rec_pool, 0, pool * sizeof(float), s));
  NA_CUDA(cudaMemsetAsync(P.d_err, 0, sizeof(int), s));
  // medium -> storage layout (device to device), then update coefficients
  for (int i = 0; i < 2; i++) {
    cudaMemcpy3DParms mp = {};
    mp.srcPtr = make_cudaPitchedPtr((void *)(i == 0 ? invK : rho), (size_t)d.nz * sizeof(float), d.nz, 1);
    mp.dstPtr = make_cudaPitchedPtr((void *)P.mod[i], (size_t)P.NZP * sizeof(float), P.NZP, 1);
    mp.dstPos = make_cudaPos((size_t)ZOFF * sizeof(float), 0, XOFF);
    mp.extent = make_cudaExtent((size_t)d.nz * sizeof(float), 1, d.nx);
    mp.kind = cudaMemcpyDeviceToDevice;
    NA_CUDA(cudaMemcpy3DAsync(&mp, s));
  }
  // the static host staging is reused by the next call: wait for the uploads
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return nfail(GPI_E_CUDA, cudaGetErrorString(e));
  rc = compute_coefficients(&P);
  for (int it = 1; !rc && it <= d.nt; it++) {
    rc = aux_step(&P, it, GPI_FORWARD);
    if (!rc) rc = step_acoustic2d(&P, 1, it, GPI_FORWARD, 0);
  }
  if (!rc) rc = aux_step(&P, d.nt + 1, GPI_FORWARD);  // velocity records of the last step
  int64_t off = 0;
  for (int k = 0; !rc && k < nrf; k++) {
    rc = transpose_records(&P, records[k], P.rec_pool + off, d.nt, nr[k]);
    off += (int64_t)nr[k] * d.nt;
  }
  if (rc) return nfail(rc, P.err.c_str());
  // a bounded pipeline wait that gave up sets the flag and leaves the
  // records incomplete: report it instead of returning success
  NA_CUDA(cudaMemcpyAsync(&h_err, P.d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  NA_CUDA(cudaStreamSynchronize(s));
  if (h_err) return nfail(GPI_E_CUDA, "a step kernel's pipeline wait timed out (records incomplete)");
  e = cudaGetLastError();
  if (e != cudaSuccess) return nfail(GPI_E_CUDA, cudaGetErrorString(e));
  return GPI_OK;
}
