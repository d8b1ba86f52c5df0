// gpi_plan.cu -- plan lifecycle and the C ABI of libgpi_fdtd.so.
//
// The plan is the device-side twin of the reference's PFdtd: P_common's
// coefficient arrays (src/fdtd/types.jl:133-166) plus, for every
// supersource, the per-worker wavefields, CPML memory and records
// (src/fdtd/types.jl:8-22, :81-88).  Shots are batched inside each launch
// instead of being looped over by Distributed workers.
#include <algorithm>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gpi_internal.cuh"

namespace gpi {

static thread_local std::string g_create_err;

int fail(Plan *p, int code, const std::string &msg) {
  if (p)
    p->err = msg;
  else
    g_create_err = msg;
  return code;
}

// Stream-ordered device allocations and uploads on the plan's stream: no
// device-wide synchronisation, so plans of other requests keep running.
// They come from one memory pool per device owned by the engine, which
// keeps freed memory for the next plan: a pool that returns memory to the
// system at a stream synchronisation (the default pool's behaviour) makes
// that synchronisation wait for every stream of the device, so one request
// finishing would stall all the others.  The pool is trimmed when the last
// plan of its device is destroyed.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[64] = {};
static int g_live[64] = {};

static cudaMemPool_t engine_pool(int dev) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (dev < 0 || dev >= 64) return nullptr;
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pools[dev] = pool;
  }
  return g_pools[dev];
}

// a stream-ordered allocation from the engine's pool of the current device
// (the device's default pool if the engine's could not be created)
cudaError_t pool_alloc(void **ptr, size_t bytes, cudaStream_t st) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPool_t pool = engine_pool(dev);
  return pool ? cudaMallocFromPoolAsync(ptr, bytes, pool, st) : cudaMallocAsync(ptr, bytes, st);
}

static void plan_born(int dev) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (dev >= 0 && dev < 64) g_live[dev]++;
}
// the last plan of a device gives the pool's memory back (once its own
// frees, ordered on its stream, have run)
static void plan_gone(int dev, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (dev < 0 || dev >= 64) return;
  if (--g_live[dev] == 0 && g_pools[dev]) {
    if (st) cudaStreamSynchronize(st);
    cudaMemPoolTrimTo(g_pools[dev], 0);
  }
}

static cudaError_t dalloc(Plan &p, void **ptr, size_t bytes) { return pool_alloc(ptr, bytes, p.stream); }
static cudaError_t h2d(Plan &p, void *dst, const void *src, size_t bytes) {
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, p.stream);
}

// ---------------------------------------------------------------------------
// derivative-field tables (get_mgrid shapes, src/fields.jl:92-671)
// ---------------------------------------------------------------------------
enum { KF = 0, KV = 1, KH = 2, KI = 3 };
static const DerivSpec DA2[] = {{2, KI, KF, KH}, {0, KH, KF, KI}, {2, KF, KF, KF}, {0, KF, KF, KF}};
static const DerivSpec DE2[] = {{2, KI, KF, KH}, {2, KH, KF, KI}, {0, KH, KF, KI}, {0, KI, KF, KH},
                                {2, KF, KF, KF}, {0, KF, KF, KF}, {0, KH, KF, KH}, {2, KH, KF, KH}};
static const DerivSpec DA3[] = {{2, KI, KI, KH}, {1, KI, KH, KI}, {0, KH, KI, KI},
                                {2, KF, KF, KF}, {1, KF, KF, KF}, {0, KF, KF, KF}};
static const DerivSpec DE3[] = {{2, KI, KI, KH}, {2, KI, KH, KI}, {2, KH, KI, KI}, {1, KI, KH, KI},
                                {1, KI, KI, KH}, {1, KH, KI, KI}, {0, KH, KI, KI}, {0, KI, KH, KI},
                                {0, KI, KI, KH}, {2, KF, KF, KF}, {1, KF, KF, KF}, {0, KF, KF, KF},
                                {1, KI, KH, KH}, {0, KH, KI, KH}, {2, KI, KH, KH}, {0, KH, KH, KI},
                                {2, KH, KI, KH}, {1, KH, KH, KI}};

int deriv_specs(int physics, int ndim, const DerivSpec **out) {
  if (physics == GPI_ACOUSTIC) {
    *out = ndim == 2 ? DA2 : DA3;
    return ndim == 2 ? 4 : 6;
  }
  *out = ndim == 2 ? DE2 : DE3;
  return ndim == 2 ? 8 : 18;
}

static const int FK[NFIELD][3] = {{KF, KF, KF}, {KF, KF, KV}, {KF, KV, KF}, {KV, KF, KF}, {KF, KF, KF},
                                  {KF, KF, KF}, {KF, KF, KF}, {KI, KH, KH}, {KH, KI, KH}, {KH, KH, KI}};
void field_kinds(int f, int *kz, int *ky, int *kx) {
  *kz = FK[f][0];
  *ky = FK[f][1];
  *kx = FK[f][2];
}
int nkind(int kind, int n, int h) {
  switch (kind) {
    case KV: return n + h;
    case KH: return n - h;
    case KI: return n - 2 * h;
    default: return n;
  }
}
static void field_shape(const Plan &p, int f, int n[3]) {
  n[0] = nkind(FK[f][0], p.d.nz, p.h);
  n[1] = p.d.ndim == 3 ? nkind(FK[f][1], p.d.ny, p.h) : 1;
  n[2] = nkind(FK[f][2], p.d.nx, p.h);
}
static int64_t field_len(const Plan &p, int f) {
  int n[3];
  field_shape(p, f, n);
  return (int64_t)n[0] * n[1] * n[2];
}

static int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// tiling of the step kernels: z-blocks of TZ rows, (3-D: TY planes),
// x-chunks of L columns; the chunk count is chosen so that the grid is a
// near multiple of the 152 SMs.
static void choose_tiling(Plan &p) {
  const int sms = 152;
  if (p.d.ndim == 2) {
    p.TZ = TZ2;
    p.TY = 1;
    p.nzb = (p.d.nz + p.TZ - 1) / p.TZ;
    p.nyb = 1;
    // interior blocks resident at once (128 threads; shared memory:
    // acoustic 33 KB, elastic 37 KB per block)
    int resident = sms * 6;
    int per_chunk = p.nzb * p.d.nshots;
    int best = 1;
    double best_eff = 0;
    // chunks of at least 16 columns (3 of them recomputed halo); grids too
    // small to fill the GPU with such chunks take chunks down to 8 columns,
    // which halves the column march a step waits for
    const int minw = (int64_t)std::max(1, p.d.nx / 16) * per_chunk < resident ? 8 : 16;
    for (int m = 1; m <= std::max(1, p.d.nx / minw); m++) {
      int64_t blocks = (int64_t)m * per_chunk;
      double waves = (double)blocks / resident;
      double eff = waves / std::ceil(waves);
      int L = (p.d.nx + m - 1) / m;
      double halo = 3.0 / L;  // redundant velocity columns
      eff *= (1.0 - halo);
      if (blocks < resident / 2) eff *= (double)blocks / (resident / 2);
      if (eff > best_eff + 1e-9) {
        best_eff = eff;
        best = m;
      }
    }
    p.xcut.assign(best + 2 * p.d.npml + 8, 0);
    p.nxb = make_xcuts(p.d.nx, best, p.d.npml, p.d.pml_faces & GPI_XMIN, p.d.pml_faces & GPI_XMAX, p.xcut.data());
    p.xcut.resize(p.nxb + 1);
    p.L = (p.d.nx + best - 1) / best;
  } else {
    p.TZ = 32;
    p.TY = 8;
    p.nzb = (p.d.nz + p.TZ - 1) / p.TZ;
    p.nyb = (p.d.ny + p.TY - 1) / p.TY;
    int per_chunk = p.nzb * p.nyb * p.d.nshots;
    int resident = sms * 6;
    int best = 1;
    double best_eff = 0;
    for (int nxb = 1; nxb <= std::max(1, p.d.nx / 16); nxb++) {
      int64_t blocks = (int64_t)nxb * per_chunk;
      double waves = (double)blocks / resident;
      double eff = waves / std::ceil(waves);
      int L = (p.d.nx + nxb - 1) / nxb;
      eff *= (1.0 - 3.0 / L);
      if (blocks < resident / 2) eff *= (double)blocks / (resident / 2);
      if (eff > best_eff + 1e-9) {
        best_eff = eff;
        best = nxb;
      }
    }
    p.nxb = best;
    p.L = (p.d.nx + best - 1) / best;
    p.nxb = (p.d.nx + p.L - 1) / p.L;
  }
}

static int64_t psi_len(const Plan &p, int axis) {
  const int64_t w = 2 * (int64_t)p.d.npml;
  if (p.d.ndim == 2) return axis == 2 ? w * p.NZP : (int64_t)p.NXP * p.zsw;
  if (axis == 2) return w * p.NYP * p.NZP;
  if (axis == 1) return (int64_t)p.NXP * w * p.NZP;
  return (int64_t)p.NXP * p.NYP * w;
}

static int nsaved(const Plan &p, int *ids) {
  if (p.d.physics == GPI_ACOUSTIC) {
    ids[0] = GPI_P;
    return 1;
  }
  ids[0] = GPI_TAUXX;
  ids[1] = GPI_TAUXZ;
  ids[2] = GPI_TAUZZ;
  return 3;
}

// with `bytes_only`, the device bytes of the plan's pool (no allocation)
int create(const gpi_plan_desc *desc, gpi_plan **out, size_t *bytes_only = nullptr) {
  if (!desc || (!out && !bytes_only)) return fail(nullptr, GPI_E_INVALID, "null argument");
  if (out) *out = nullptr;
  const gpi_plan_desc &d = *desc;
  if (d.physics != GPI_ACOUSTIC && d.physics != GPI_ELASTIC) return fail(nullptr, GPI_E_INVALID, "physics");
  if (d.ndim != 2 && d.ndim != 3) return fail(nullptr, GPI_E_INVALID, "ndim must be 2 or 3");
  if (d.order != 2 && d.order != 4 && d.order != 6 && d.order != 8)
    return fail(nullptr, GPI_E_INVALID, "order must be 2, 4, 6 or 8");
  // orders other than 4 (k_generic.cu): forward modelling only
  if (d.order != 4 && (d.npw != 1 || d.checkpoints > 0))
    return fail(nullptr, GPI_E_UNSUPPORTED, "stencil orders 2, 6, 8: forward runs only (npw = 1)");
  if (d.order != 4 && d.nshots > 65535)
    return fail(nullptr, GPI_E_UNSUPPORTED, "stencil orders 2, 6, 8: at most 65535 shots per plan");
  if (d.nt < 1 || d.nshots < 1 || (d.npw != 1 && d.npw != 2)) return fail(nullptr, GPI_E_INVALID, "nt/nshots/npw");
  if (d.checkpoints < 0 || (d.checkpoints > 0 && d.npw != 2))
    return fail(nullptr, GPI_E_INVALID, "checkpoints: > 0 only with npw = 2");
  if (d.checkpoints > 0 && d.physics != GPI_ACOUSTIC && (d.ndim != 3 || (d.free_faces & GPI_ZMIN)))
    return fail(nullptr, GPI_E_UNSUPPORTED,
                "checkpointed gradients: acoustic media, or 3-D elastic media without a free surface");
  if (d.npml < 1 || d.nbound < 1) return fail(nullptr, GPI_E_INVALID, "npml/nbound");
  if (d.imaging != 0 && d.imaging != 1) return fail(nullptr, GPI_E_INVALID, "imaging must be 0 or 1");
  if (!(d.dt > 0) || !(d.dz > 0) || !(d.dx > 0) || (d.ndim == 3 && !(d.dy > 0)))
    return fail(nullptr, GPI_E_INVALID, "dt and grid steps must be positive");
  const int h = d.order - 1;
  const int ny = d.ndim == 3 ? d.ny : 1;
  // CPML strips of the min and max faces must not overlap on any derivative
  // field (the shortest derivative axis is n - 2h).
  {
    const int n3[3] = {d.nz, ny, d.nx};
    const int lo3[3] = {GPI_ZMIN, GPI_YMIN, GPI_XMIN}, hi3[3] = {GPI_ZMAX, GPI_YMAX, GPI_XMAX};
    for (int ax = 0; ax < 3; ax++) {
      if (ax == 1 && d.ndim == 2) continue;
      const int strips = ((d.pml_faces & lo3[ax]) ? 1 : 0) + ((d.pml_faces & hi3[ax]) ? 1 : 0);
      if (n3[ax] - 2 * h < strips * d.npml + 1)
        return fail(nullptr, GPI_E_INVALID, "grid too small for its PML strips");
    }
  }
  gpi_plan *pl = new gpi_plan();
  Plan &p = pl->p;
  p.d = d;
  p.d.ny = ny;
  p.d.rigid_faces |= d.pml_faces;  // fdtd.jl:215: rigid U pml
  p.h = h;
  cudaGetDevice(&p.device);
  p.nder = deriv_specs(d.physics, d.ndim, &p.ds);
  p.present[GPI_VX] = p.present[GPI_VZ] = 1;
  if (d.ndim == 3) p.present[GPI_VY] = 1;
  if (d.physics == GPI_ACOUSTIC)
    p.present[GPI_P] = 1;
  else {
    p.present[GPI_TAUXX] = p.present[GPI_TAUZZ] = p.present[GPI_TAUXZ] = 1;
    if (d.ndim == 3) p.present[GPI_TAUYY] = p.present[GPI_TAUXY] = p.present[GPI_TAUYZ] = 1;
  }
  choose_tiling(p);
  p.NZP = (int)round_up((int64_t)p.nzb * p.TZ + 2 * ZOFF + 4, 32);
  p.NXP = d.nx + h + 2 * XOFF + 4;
  p.NYP = d.ndim == 3 ? (int)(p.nyb * p.TY + 2 * YOFF + 4) : 1;
  p.fstride = (int64_t)p.NZP * p.NYP * p.NXP;
  if (d.ndim == 2) {
    p.zsw = zstrip_stride(d.npml);
    p.pzw = zstrip_window(p.nzb, p.TZ, d.nz, d.npml, d.pml_faces & GPI_ZMIN, d.pml_faces & GPI_ZMAX);
  }

  // ---- pool layout ----
  std::vector<std::pair<float **, int64_t>> allocs;
  int nf = 0;
  for (int f = 0; f < NFIELD; f++) nf += p.present[f];
  for (int b = 0; b < 2; b++)
    for (int ipw = 0; ipw < d.npw; ipw++)
      for (int f = 0; f < NFIELD; f++)
        if (p.present[f]) allocs.push_back({&p.state[b][ipw][f], p.fstride * d.nshots});
  for (int q = 0; q < p.nder; q++) {
    const int ax = p.ds[q].axis;
    const int fmin = ax == 0 ? GPI_ZMIN : ax == 1 ? GPI_YMIN : GPI_XMIN;
    const int fmax = ax == 0 ? GPI_ZMAX : ax == 1 ? GPI_YMAX : GPI_XMAX;
    if (!(d.pml_faces & (fmin | fmax))) continue;
    p.psi_stride[q] = psi_len(p, ax);
    for (int b = 0; b < 2; b++)
      for (int ipw = 0; ipw < d.npw; ipw++) allocs.push_back({&p.psi[b][ipw][q], p.psi_stride[q] * d.nshots});
  }
  p.nmod = d.physics == GPI_ACOUSTIC ? 2 : 3;
  p.ncoef = d.physics == GPI_ACOUSTIC ? d.ndim + 1 : (d.ndim == 2 ? 5 : 8);
  for (int i = 0; i < p.nmod; i++) allocs.push_back({&p.mod[i], p.fstride});
  {
    // get_fc (src/fdtd/fdtd.jl:313-332): 1 / (den * d) in FP64, stored as FP32
    const double den = d.order == 4 ? 24.0 : d.order == 6 ? 1920.0 : d.order == 8 ? 107520.0 : 1.0;
    p.gdsI[0] = (float)(1.0 / (d.dz * den));
    p.gdsI[1] = d.ndim == 3 ? (float)(1.0 / (d.dy * den)) : 0.f;
    p.gdsI[2] = (float)(1.0 / (d.dx * den));
  }
  for (int i = 0; i < p.ncoef; i++) allocs.push_back({&p.coef[i], p.fstride});
  allocs.push_back({&p.pml, (int64_t)p.nder * 3 * 2 * d.npml});
  allocs.push_back({(float **)&p.d_err, 64});
  allocs.push_back({(float **)&p.d_it, 64});
  if (d.npw == 2 && d.checkpoints > 0) {
    // checkpointed adjoint: state slots instead of the boundary store
    for (int i = 0; i < p.nmod; i++) allocs.push_back({&p.grad[i], p.fstride * d.nshots});
    p.ck_slots = d.checkpoints;
    p.ck_floats = ckpt_slot_floats(p);
    allocs.push_back({&p.ck_pool, p.ck_floats * p.ck_slots});
  } else if (d.npw == 2) {
    for (int i = 0; i < p.nmod && i < 2; i++) allocs.push_back({&p.grad[i], p.fstride * d.nshots});
    if (d.physics == GPI_ACOUSTIC && d.ndim == 2)
      for (int i = 0; i < 2; i++) allocs.push_back({&p.img[i], p.fstride * d.nshots});
    int ids[3];
    int ns = nsaved(p, ids);
    p.bstep = 0;
    p.bsnap = 0;
    for (int q = 0; q < ns; q++) {
      int n[3];
      field_shape(p, ids[q], n);
      for (int ax = 0; ax < 3; ax++) {
        if (ax == 1 && d.ndim == 2) continue;
        int64_t s = 2 * (int64_t)d.nbound;
        for (int o = 0; o < 3; o++)
          if (o != ax) s *= n[o];
        p.bstep += s;
      }
      p.bsnap += p.fstride;
    }
    p.bsnap += p.fstride * (d.ndim == 3 ? 3 : 2);
    allocs.push_back({&p.bstore, (p.bstep * d.nt + p.bsnap) * d.nshots});
    allocs.push_back({&p.bprev, p.bstep * d.nshots});
  }
  size_t total = 0;
  for (auto &a : allocs) total += (size_t)round_up(a.second, 64) * sizeof(float);
  if (bytes_only) {
    *bytes_only = total;
    delete pl;
    return GPI_OK;
  }
  // one stream-ordered allocation (set-up stream, synchronised below)
  cudaStream_t cs = nullptr;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
    delete pl;
    cudaGetLastError();
    return fail(nullptr, GPI_E_CUDA, "stream creation failed");
  }
  cudaError_t e = pool_alloc(&p.pool, total, cs);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cs);
    delete pl;
    cudaGetLastError();
    return fail(nullptr, GPI_E_NOMEM, "allocation of " + std::to_string(total) + " bytes failed");
  }
  p.pool_bytes = total;
  char *c = (char *)p.pool;
  for (auto &a : allocs) {
    *a.first = (float *)c;
    c += (size_t)round_up(a.second, 64) * sizeof(float);
  }
  // zeroed state, identity PML (kI = 1) until gpi_set_pml is called
  std::vector<float> pm((size_t)p.nder * 3 * 2 * d.npml, 0.f);
  for (int q = 0; q < p.nder; q++)
    for (int i = 0; i < 2 * d.npml; i++) {
      pm[((size_t)q * 3 + 1) * 2 * d.npml + i] = 1.f;
      pm[((size_t)q * 3 + 2) * 2 * d.npml + i] = 1.f;
    }
  e = cudaMemsetAsync(p.pool, 0, total, cs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(p.pml, pm.data(), pm.size() * sizeof(float), cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) {
    cudaFreeAsync(p.pool, cs);
    cudaStreamSynchronize(cs);
    cudaStreamDestroy(cs);
    delete pl;
    return fail(nullptr, GPI_E_CUDA, cudaGetErrorString(e));
  }
  cudaStreamDestroy(cs);
  p.rec_n.assign(d.nshots, std::vector<int>(NFIELD, 0));
  p.rec_cp.assign(d.nshots, std::vector<std::vector<int64_t>>(NFIELD));
  p.rec_off.assign(d.nshots, std::vector<std::vector<int64_t>>(NFIELD));
  p.rec_w.assign(d.nshots, std::vector<std::vector<float>>(NFIELD));
  p.rec_base.assign(d.nshots, std::vector<int64_t>(NFIELD, -1));
  p.src.assign(2, std::vector<std::vector<Plan::Src>>(d.nshots, std::vector<Plan::Src>(NFIELD)));
  p.adj_dev.assign(d.nshots, std::vector<float *>(NFIELD, nullptr));
  {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    bool ok = cudaEventCreateWithFlags(&p.ev_fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < Plan::NSIDE; k++)
      ok = ok && cudaStreamCreateWithPriority(&p.side[k], cudaStreamNonBlocking, hi) == cudaSuccess &&
           cudaEventCreateWithFlags(&p.ev_join[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      // every step kernel then runs on the plan stream
      cudaGetLastError();
      if (p.ev_fork) cudaEventDestroy(p.ev_fork);
      for (int k = 0; k < Plan::NSIDE; k++) {
        if (p.side[k]) cudaStreamDestroy(p.side[k]);
        if (p.ev_join[k]) cudaEventDestroy(p.ev_join[k]);
        p.side[k] = nullptr;
        p.ev_join[k] = nullptr;
      }
      p.ev_fork = nullptr;
    }
  }
  plan_born(p.device);
  *out = pl;
  return GPI_OK;
}

int fork_side(Plan *p, int nside, cudaStream_t *out) {
  for (int k = 0; k < nside; k++) out[k] = p->stream;
  if (nside == 0 || !p->side[0]) return GPI_OK;
  GPI_CUDA(p, cudaEventRecord(p->ev_fork, p->stream));
  for (int k = 0; k < nside; k++) {
    GPI_CUDA(p, cudaStreamWaitEvent(p->side[k], p->ev_fork, 0));
    out[k] = p->side[k];
  }
  return GPI_OK;
}
int join_side(Plan *p, int nside) {
  if (nside == 0 || !p->side[0]) return GPI_OK;
  for (int k = 0; k < nside; k++) {
    GPI_CUDA(p, cudaEventRecord(p->ev_join[k], p->side[k]));
    GPI_CUDA(p, cudaStreamWaitEvent(p->stream, p->ev_join[k], 0));
  }
  return GPI_OK;
}

static void free_dev(Plan &p, void *&x) {
  if (x) cudaFreeAsync(x, p.stream);
  x = nullptr;
}

static void free_sources(Plan &p) {
  free_dev(p, (void *&)p.d_cells);
  free_dev(p, (void *&)p.d_pair_j);
  free_dev(p, (void *&)p.d_pair_w);
  free_dev(p, (void *&)p.d_wav);
  free_dev(p, (void *&)p.d_wav_ns);
  free_dev(p, (void *&)p.d_amount);
  free_dev(p, (void *&)p.d_group_ptr);
  free_dev(p, (void *&)p.d_tiles);
  p.h_cells.clear();
  for (auto b : p.wav_bufs) cudaFreeAsync(b, p.stream);
  p.wav_bufs.clear();
  p.n_cells = 0;
}
static void free_receivers(Plan &p) {
  free_dev(p, (void *&)p.rec_pool);
  free_dev(p, (void *&)p.d_rtask);
  free_dev(p, (void *&)p.d_roff);
  free_dev(p, (void *&)p.d_rw);
  p.n_rtask = 0;
}

void destroy(gpi_plan *pl) {
  if (!pl) return;
  Plan &p = pl->p;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaSetDevice(p.device);
  if (p.stream) cudaStreamSynchronize(p.stream);
  drop_graphs(p);
  for (int k = 0; k < Plan::NSIDE; k++) {
    if (p.side[k]) {
      cudaStreamSynchronize(p.side[k]);
      cudaStreamDestroy(p.side[k]);
    }
    if (p.ev_join[k]) cudaEventDestroy(p.ev_join[k]);
  }
  if (p.ev_fork) cudaEventDestroy(p.ev_fork);
  // stream-ordered frees on the plan's stream, then its own stream if any
  free_sources(p);
  free_receivers(p);
  for (auto &row : p.adj_dev)
    for (float *&d : row)
      if (d) cudaFreeAsync(d, p.stream), d = nullptr;
  {
    void *sb = p.snap_buf;
    free_dev(p, sb);
    p.snap_buf = nullptr;
    void *il = p.illum;
    free_dev(p, il);
    p.illum = nullptr;
    void *bb = p.born;
    free_dev(p, bb);
    p.born = nullptr;
  }
  free_dev(p, p.pool);
  plan_gone(p.device, p.stream);
  if (p.own_stream) cudaStreamDestroy(p.own_stream);
  cudaSetDevice(dev);
  delete pl;
}

// ---------------------------------------------------------------------------
// medium and PML
// ---------------------------------------------------------------------------
static int to_storage(Plan &p, float *dst, const float *src, int n1, int n2, int n3, int on_device) {
  // column-major (n1, n2, n3) -> padded storage
  cudaMemcpy3DParms m = {};
  m.srcPtr = make_cudaPitchedPtr((void *)src, (size_t)n1 * sizeof(float), n1, n2);
  m.dstPtr = make_cudaPitchedPtr((void *)dst, (size_t)p.NZP * sizeof(float), p.NZP, p.NYP);
  m.srcPos = make_cudaPos(0, 0, 0);
  m.dstPos = make_cudaPos((size_t)ZOFF * sizeof(float), p.d.ndim == 3 ? YOFF : 0, XOFF);
  m.extent = make_cudaExtent((size_t)n1 * sizeof(float), n2, n3);
  m.kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  GPI_CUDA(&p, cudaMemcpy3DAsync(&m, p.stream));
  return GPI_OK;
}
static int from_storage(Plan &p, float *dst, const float *src, int n1, int n2, int n3, int on_device) {
  cudaMemcpy3DParms m = {};
  m.srcPtr = make_cudaPitchedPtr((void *)src, (size_t)p.NZP * sizeof(float), p.NZP, p.NYP);
  m.dstPtr = make_cudaPitchedPtr((void *)dst, (size_t)n1 * sizeof(float), n1, n2);
  m.srcPos = make_cudaPos((size_t)ZOFF * sizeof(float), p.d.ndim == 3 ? YOFF : 0, XOFF);
  m.dstPos = make_cudaPos(0, 0, 0);
  m.extent = make_cudaExtent((size_t)n1 * sizeof(float), n2, n3);
  m.kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  GPI_CUDA(&p, cudaMemcpy3DAsync(&m, p.stream));
  return GPI_OK;
}

int set_medium(Plan &p, const float *const *mod, int on_device) {
  if (!mod) return fail(&p, GPI_E_INVALID, "mod is null");
  for (int i = 0; i < p.nmod; i++) {
    if (!mod[i]) return fail(&p, GPI_E_INVALID, "mod array missing");
    int rc = to_storage(p, p.mod[i], mod[i], p.d.nz, p.d.ny, p.d.nx, on_device);
    if (rc) return rc;
  }
  int rc = compute_coefficients(&p);
  if (rc) return rc;
  if (!on_device) GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  p.src_dirty = true;  // injection scaling reads rho / dtK at run time, nothing to redo
  return GPI_OK;
}

// update!(pa, medium, medium_pert) for Born plans: the perturbations, kept
// in storage layout; the secondary-source ratios are formed from them and
// the current medium at the start of each Born run (k_born.cu)
int set_born(Plan &p, const float *const *dmod, int on_device) {
  if (p.d.physics != GPI_ACOUSTIC || p.d.ndim != 2 || p.d.npw != 2)
    return fail(&p, GPI_E_UNSUPPORTED, "Born modelling: 2-D acoustic plans with npw = 2");
  if (!dmod || !dmod[0] || !dmod[1]) return fail(&p, GPI_E_INVALID, "dmod arrays");
  if (!p.born) {
    if (pool_alloc((void **)&p.born, 5 * p.fstride * sizeof(float), p.stream) != cudaSuccess) {
      cudaGetLastError();
      p.born = nullptr;
      return fail(&p, GPI_E_NOMEM, "Born perturbation buffers");
    }
    GPI_CUDA(&p, cudaMemsetAsync(p.born, 0, 5 * p.fstride * sizeof(float), p.stream));
  }
  for (int i = 0; i < 2; i++) {
    int rc = to_storage(p, p.born + (3 + i) * p.fstride, dmod[i], p.d.nz, 1, p.d.nx, on_device);
    if (rc) return rc;
  }
  if (!on_device) GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  p.have_born = true;
  return GPI_OK;
}

int set_pml(Plan &p, int q, int len, const float *a, const float *b, const float *kI) {
  if (q < 0 || q >= p.nder || !a || !b || !kI) return fail(&p, GPI_E_INVALID, "pml field index or null array");
  if (len != 2 * p.d.npml) return fail(&p, GPI_E_INVALID, "pml arrays must hold 2*npml values");
  const size_t n = 2 * (size_t)p.d.npml;
  float *dst = p.pml + (size_t)q * 3 * n;
  GPI_CUDA(&p, cudaMemcpyAsync(dst, a, n * sizeof(float), cudaMemcpyHostToDevice, p.stream));
  GPI_CUDA(&p, cudaMemcpyAsync(dst + n, b, n * sizeof(float), cudaMemcpyHostToDevice, p.stream));
  GPI_CUDA(&p, cudaMemcpyAsync(dst + 2 * n, kI, n * sizeof(float), cudaMemcpyHostToDevice, p.stream));
  GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  return GPI_OK;
}

// ---------------------------------------------------------------------------
// sources and receivers
// ---------------------------------------------------------------------------
static bool is_vel(int f) { return f == GPI_VX || f == GPI_VY || f == GPI_VZ; }
static bool is_stress_src(int f) { return f == GPI_P || f == GPI_TAUXX || f == GPI_TAUYY || f == GPI_TAUZZ; }
static int kind_of(int f) { return f == GPI_VX ? 0 : f == GPI_VY ? 1 : f == GPI_VZ ? 2 : 3; }

static int check_csc(Plan &p, int field, int n, const int64_t *cp, const int64_t *rv) {
  if (field < 0 || field >= NFIELD || !p.present[field]) return fail(&p, GPI_E_INVALID, "field not part of this physics");
  if (n < 0 || (n > 0 && (!cp || !rv))) return fail(&p, GPI_E_INVALID, "csc arrays");
  const int64_t len = field_len(p, field);
  if (n > 0 && cp[0] != 0) return fail(&p, GPI_E_INVALID, "colptr[0] must be 0");
  for (int j = 0; j < n; j++) {
    if (cp[j + 1] < cp[j]) return fail(&p, GPI_E_INVALID, "colptr not monotone");
    for (int64_t k = cp[j]; k < cp[j + 1]; k++)
      if (rv[k] < 0 || rv[k] >= len) return fail(&p, GPI_E_INVALID, "row index outside the field");
  }
  return GPI_OK;
}

// the device wavelets of an adjoint source set by set_adjoint_l2
static void drop_adj(Plan &p, int shot, int field) {
  if (p.adj_dev.empty()) return;
  float *&d = p.adj_dev[shot][field];
  if (d) cudaFreeAsync(d, p.stream);
  d = nullptr;
}

int set_sources(Plan &p, int ipw, int shot, int field, int ns, const int64_t *cp, const int64_t *rv, const float *nz,
                const float *wav) {
  if (ipw < 1 || ipw > p.d.npw) return fail(&p, GPI_E_INVALID, "ipw");
  if (shot < 0 || shot >= p.d.nshots) return fail(&p, GPI_E_INVALID, "shot index");
  if (field < 0 || field >= NFIELD || !p.present[field]) return fail(&p, GPI_E_INVALID, "source field not in this physics");
  if (ns < 0 || (ns > 0 && !wav)) return fail(&p, GPI_E_INVALID, "wavelets");
  Plan::Src &s = p.src[ipw - 1][shot][field];
  s = Plan::Src();
  if (ipw == 2) drop_adj(p, shot, field);
  if (ipw == 1) {
    if (!is_vel(field) && !is_stress_src(field)) return fail(&p, GPI_E_INVALID, "sources act on p, tauii or velocities");
    int rc = check_csc(p, field, ns, cp, rv);
    if (rc) return rc;
    if (ns > 0 && !nz) return fail(&p, GPI_E_INVALID, "nzval");
    s.cp.assign(cp, cp + ns + 1);
    s.rv.assign(rv, rv + (ns ? cp[ns] : 0));
    s.nz.assign(nz, nz + (ns ? cp[ns] : 0));
  } else {
    // adjoint wavefield: injected through rinterpolatew of `field`
    // (add_velocity_source!, src/fdtd/source.jl:141-156, velocities only)
    if (!is_vel(field)) return fail(&p, GPI_E_UNSUPPORTED, "adjoint sources act on velocity fields only");
    if (p.rec_n[shot][field] != ns) return fail(&p, GPI_E_STATE, "adjoint sources need the receivers of that field first");
  }
  s.ns = ns;
  s.wav.assign(wav, wav + (size_t)ns * p.d.nt);
  p.src_dirty = true;
  return GPI_OK;
}

static int check_err(Plan &p);

// The adjoint sources of gradient! with L2DistLoss for one shot and
// receiver field, computed on the device from the records of the last run
// (src/fdtd/func_grad.jl:11-49: deriv(L2DistLoss(), dobs, dcal) =
// 2 (dobs - dcal), reverse!, injected through the receiver interpolation);
// *misfit = sum (dobs - dcal)^2 (value(L2DistLoss(), dobs, dcal)).
int set_adjoint_l2(Plan &p, int shot, int field, const float *dobs, int on_device, double *misfit) {
  if (p.d.npw != 2) return fail(&p, GPI_E_INVALID, "adjoint sources need npw = 2");
  if (shot < 0 || shot >= p.d.nshots || field < 0 || field >= NFIELD) return fail(&p, GPI_E_INVALID, "shot/field");
  if (!is_vel(field)) return fail(&p, GPI_E_UNSUPPORTED, "adjoint sources act on velocity fields only");
  const int nr = p.rec_n[shot][field];
  if (nr <= 0 || p.rec_base[shot][field] < 0 || !p.rec_pool)
    return fail(&p, GPI_E_STATE, "no records of this shot and field (run forward_save first)");
  if (!dobs || !misfit) return fail(&p, GPI_E_INVALID, "null argument");
  const int nt = p.d.nt;
  const size_t n = (size_t)nt * nr;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != p.device) GPI_CUDA(&p, cudaSetDevice(p.device));
  p.src[1][shot][field] = Plan::Src();
  drop_adj(p, shot, field);
  float *adj = nullptr, *tmp = nullptr;
  double *part = nullptr;
  const int nblk = adjoint_l2_blocks(nt, nr);
  int rc = GPI_OK;
  if (pool_alloc((void **)&adj, n * sizeof(float), p.stream) != cudaSuccess ||
      pool_alloc((void **)&part, (nblk + 1) * sizeof(double), p.stream) != cudaSuccess)
    rc = fail(&p, GPI_E_NOMEM, "adjoint source buffers");
  const float *d = dobs;
  if (!rc && !on_device) {
    if (pool_alloc((void **)&tmp, n * sizeof(float), p.stream) != cudaSuccess ||
        cudaMemcpyAsync(tmp, dobs, n * sizeof(float), cudaMemcpyHostToDevice, p.stream) != cudaSuccess)
      rc = fail(&p, GPI_E_CUDA, "observed data upload");
    d = tmp;
  }
  if (!rc) rc = adjoint_l2_launch(&p, adj, part, part + nblk, d, p.rec_pool + p.rec_base[shot][field], nt, nr);
  double h = 0.0;
  if (!rc && (cudaMemcpyAsync(&h, part + nblk, sizeof(double), cudaMemcpyDeviceToHost, p.stream) != cudaSuccess ||
              cudaStreamSynchronize(p.stream) != cudaSuccess))
    rc = fail(&p, GPI_E_CUDA, "misfit read");
  if (tmp) cudaFreeAsync(tmp, p.stream);
  if (part) cudaFreeAsync(part, p.stream);
  if (rc) {
    if (adj) cudaFreeAsync(adj, p.stream);
    if (dev != p.device) cudaSetDevice(dev);
    return rc;
  }
  Plan::Src &s = p.src[1][shot][field];
  s.ns = nr;
  s.on_dev = true;
  p.adj_dev[shot][field] = adj;
  p.src_dirty = true;
  *misfit = h;
  if (dev != p.device) cudaSetDevice(dev);
  return check_err(p);
}

int clear_sources(Plan &p, int ipw, int shot) {
  if (ipw < 1 || ipw > p.d.npw) return fail(&p, GPI_E_INVALID, "ipw");
  for (int s = 0; s < p.d.nshots; s++)
    if (shot < 0 || shot == s)
      for (int f = 0; f < NFIELD; f++) {
        p.src[ipw - 1][s][f] = Plan::Src();
        if (ipw == 2) drop_adj(p, s, f);
      }
  p.src_dirty = true;
  return GPI_OK;
}

// 0-based linear index of a field -> reference (r, y, c), 1-based
static void unravel(const Plan &p, int field, int64_t lin, int *r, int *y, int *c) {
  int n[3];
  field_shape(p, field, n);
  *r = (int)(lin % n[0]) + 1;
  *y = (int)((lin / n[0]) % n[1]) + 1;
  *c = (int)(lin / ((int64_t)n[0] * n[1])) + 1;
}

int set_receivers(Plan &p, int shot, int field, int nr, const int64_t *cp, const int64_t *rv, const float *nz) {
  if (shot < 0 || shot >= p.d.nshots) return fail(&p, GPI_E_INVALID, "shot index");
  int rc = check_csc(p, field, nr, cp, rv);
  if (rc) return rc;
  if (nr > 0 && !nz) return fail(&p, GPI_E_INVALID, "nzval");
  p.rec_n[shot][field] = nr;
  p.rec_cp[shot][field].assign(cp, cp + nr + 1);
  std::vector<int64_t> off;
  const int64_t nnz = nr ? cp[nr] : 0;
  off.resize(nnz);
  for (int64_t k = 0; k < nnz; k++) {
    int r, y, c;
    unravel(p, field, rv[k], &r, &y, &c);
    off[k] = soff(p, r, y, c);
  }
  p.rec_off[shot][field] = off;
  p.rec_w[shot][field].assign(nz, nz + nnz);
  p.rec_dirty = true;
  p.src_dirty = true;  // adjoint injection follows the receivers
  return GPI_OK;
}

static int compile_receivers(Plan &p) {
  free_receivers(p);
  std::vector<RecTask> tasks;
  std::vector<int64_t> offs;
  std::vector<float> ws;
  size_t pool = 0;
  for (int s = 0; s < p.d.nshots; s++)
    for (int f = 0; f < NFIELD; f++) {
      const int nr = p.rec_n[s][f];
      p.rec_base[s][f] = -1;
      if (nr <= 0) continue;
      p.rec_base[s][f] = (int64_t)pool;
      const auto &cp = p.rec_cp[s][f];
      for (int j = 0; j < nr; j++) {
        RecTask t;
        t.shot = s;
        t.field = f;
        t.e0 = (int32_t)(offs.size() + cp[j]);
        t.e1 = (int32_t)(offs.size() + cp[j + 1]);
        t.out = (int64_t)pool + j;
        t.stride = nr;
        t.pad = 0;
        tasks.push_back(t);
      }
      offs.insert(offs.end(), p.rec_off[s][f].begin(), p.rec_off[s][f].end());
      ws.insert(ws.end(), p.rec_w[s][f].begin(), p.rec_w[s][f].end());
      pool += (size_t)nr * p.d.nt;
    }
  p.rec_pool_floats = pool;
  p.n_rtask = (int)tasks.size();
  if (pool) GPI_CUDA(&p, dalloc(p, (void **)&p.rec_pool, pool * sizeof(float)));
  if (!tasks.empty()) {
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_rtask, tasks.size() * sizeof(RecTask)));
    GPI_CUDA(&p, h2d(p, p.d_rtask, tasks.data(), tasks.size() * sizeof(RecTask)));
  }
  if (!offs.empty()) {
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_roff, offs.size() * sizeof(int64_t)));
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_rw, ws.size() * sizeof(float)));
    GPI_CUDA(&p, h2d(p, p.d_roff, offs.data(), offs.size() * sizeof(int64_t)));
    GPI_CUDA(&p, h2d(p, p.d_rw, ws.data(), ws.size() * sizeof(float)));
  }
  p.rec_dirty = false;
  return GPI_OK;
}

// Turn the spray matrices into injection cells grouped by (ipw, shot, kind)
// and sorted by (column, y, row): the step kernels sweep columns in order
// and pick the cells of the current column.  Velocity cells outside the
// @inn domain are dropped, as muladd_with_density_* ignores them
// (src/fdtd/source.jl:166-177).
static int compile_sources(Plan &p) {
  free_sources(p);
  const int h = p.h;
  struct Tmp {
    InjCell c;
    std::vector<std::pair<int, float>> pairs;
  };
  std::vector<std::vector<Tmp>> groups((size_t)2 * p.d.nshots * NKIND);
  std::vector<float *> wavptr;
  std::vector<int32_t> wavns;
  for (int ipw = 0; ipw < p.d.npw; ipw++)
    for (int s = 0; s < p.d.nshots; s++)
      for (int f = 0; f < NFIELD; f++) {
        const Plan::Src &src = p.src[ipw][s][f];
        const bool dev_wav = ipw == 1 && src.on_dev;  // already on the device (set_adjoint_l2)
        if (src.ns <= 0) continue;
        const int kind = kind_of(f);
        // the adjoint wavefield takes velocity sources only: add_stress_source!
        // injects into wavefield 1 alone (src/fdtd/source.jl:61-77)
        if (ipw == 1 && kind == 3) continue;
        // spray matrix
        const std::vector<int64_t> *cp, *rows = nullptr;
        const std::vector<float> *w;
        std::vector<int64_t> lin;
        if (ipw == 0) {
          cp = &src.cp;
          rows = &src.rv;
          w = &src.nz;
        } else {
          if (p.rec_n[s][f] != src.ns) return fail(&p, GPI_E_STATE, "adjoint sources and receivers disagree");
          cp = &p.rec_cp[s][f];
          w = &p.rec_w[s][f];
          // receivers are stored as storage offsets; recover (r, y, c)
          lin.clear();
        }
        float *dw = nullptr;
        if (dev_wav) {
          dw = p.adj_dev[s][f];
        } else {
          GPI_CUDA(&p, dalloc(p, (void **)&dw, src.wav.size() * sizeof(float)));
          GPI_CUDA(&p, h2d(p, dw, src.wav.data(), src.wav.size() * sizeof(float)));
          p.wav_bufs.push_back(dw);
        }
        const int widx = (int)wavptr.size();
        wavptr.push_back(dw);
        wavns.push_back(src.ns);
        std::map<int64_t, size_t> where;  // row -> index in this projection's cells
        std::vector<Tmp> cells;
        for (int j = 0; j < src.ns; j++)
          for (int64_t k = (*cp)[j]; k < (*cp)[j + 1]; k++) {
            int r, y, c;
            int64_t key;
            if (ipw == 0) {
              unravel(p, f, (*rows)[k], &r, &y, &c);
              key = (*rows)[k];
            } else {
              // invert the storage offset of the receiver entry
              int64_t o = p.rec_off[s][f][k];
              r = (int)(o % p.NZP) - ZOFF + 1;
              int64_t rest = o / p.NZP;
              y = p.d.ndim == 3 ? (int)(rest % p.NYP) - YOFF + 1 : 1;
              c = (int)(rest / p.NYP) - XOFF + 1;
              key = o;
            }
            auto it = where.find(key);
            if (it == where.end()) {
              Tmp t;
              t.c.row = r;
              t.c.ydx = y;
              t.c.col = c;
              t.c.wav = widx;
              t.c.kind = kind;
              t.c.pad = 0;
              t.c.off = soff(p, r, y, c);
              t.c.roff0 = t.c.roff1 = 0;
              where[key] = cells.size();
              cells.push_back(t);
              it = where.find(key);
            }
            cells[it->second].pairs.push_back({j, (*w)[k]});
          }
        int n[3];
        field_shape(p, f, n);
        for (auto &t : cells) {
          if (kind < 3) {
            const int r = t.c.row, y = t.c.ydx, c = t.c.col;
            bool in = r - h >= 1 && r - h <= n[0] - 2 * h && c - h >= 1 && c - h <= n[2] - 2 * h;
            if (p.d.ndim == 3) in = in && y - h >= 1 && y - h <= n[1] - 2 * h;
            if (!in) continue;
            // @av_{x,y,z}i(rho) at the @inn cell (iz, iy, ix) = cell - h
            int z = r - h, yy = p.d.ndim == 3 ? y - h : 1, x = c - h;
            int zz = z + (kind != 2 ? h : 0), y2 = p.d.ndim == 3 ? yy + (kind != 1 ? h : 0) : 1, xx = x + (kind != 0 ? h : 0);
            t.c.roff0 = soff(p, zz, y2, xx);
            t.c.roff1 = soff(p, zz + (kind == 2), y2 + (kind == 1), xx + (kind == 0));
          }
          groups[((size_t)ipw * p.d.nshots + s) * NKIND + kind].push_back(t);
        }
      }
  std::vector<InjCell> cells;
  std::vector<int32_t> pj;
  std::vector<float> pw;
  p.group_ptr.assign(groups.size() + 1, 0);
  for (size_t g = 0; g < groups.size(); g++) {
    auto &G = groups[g];
    std::stable_sort(G.begin(), G.end(), [](const Tmp &a, const Tmp &b) {
      if (a.c.col != b.c.col) return a.c.col < b.c.col;
      if (a.c.ydx != b.c.ydx) return a.c.ydx < b.c.ydx;
      return a.c.row < b.c.row;
    });
    p.group_ptr[g] = (int32_t)cells.size();
    for (auto &t : G) {
      t.c.e0 = (int32_t)pj.size();
      for (auto &pr : t.pairs) {
        pj.push_back(pr.first);
        pw.push_back(pr.second);
      }
      t.c.e1 = (int32_t)pj.size();
      cells.push_back(t.c);
    }
  }
  p.group_ptr[groups.size()] = (int32_t)cells.size();
  p.n_cells = (int)cells.size();
  // a cell twice in a group (two stress source fields on one cell) needs
  // the in-order injection
  p.inj_shared = false;
  for (size_t g = 0; g + 1 < p.group_ptr.size() && !p.inj_shared; g++) {
    std::vector<int64_t> offs;
    for (int32_t k = p.group_ptr[g]; k < p.group_ptr[g + 1]; k++) offs.push_back(cells[k].off);
    std::sort(offs.begin(), offs.end());
    p.inj_shared = std::adjacent_find(offs.begin(), offs.end()) != offs.end();
  }
  p.h_cells = cells;
  GPI_CUDA(&p, dalloc(p, (void **)&p.d_group_ptr, p.group_ptr.size() * sizeof(int32_t)));
  GPI_CUDA(&p, h2d(p, p.d_group_ptr, p.group_ptr.data(), p.group_ptr.size() * sizeof(int32_t)));
  if (p.n_cells) {
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_cells, cells.size() * sizeof(InjCell)));
    GPI_CUDA(&p, h2d(p, p.d_cells, cells.data(), cells.size() * sizeof(InjCell)));
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_pair_j, pj.size() * sizeof(int32_t)));
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_pair_w, pw.size() * sizeof(float)));
    GPI_CUDA(&p, h2d(p, p.d_pair_j, pj.data(), pj.size() * sizeof(int32_t)));
    GPI_CUDA(&p, h2d(p, p.d_pair_w, pw.data(), pw.size() * sizeof(float)));
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_amount, cells.size() * sizeof(float)));
  }
  if (!wavptr.empty()) {
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_wav, wavptr.size() * sizeof(float *)));
    GPI_CUDA(&p, dalloc(p, (void **)&p.d_wav_ns, wavns.size() * sizeof(int32_t)));
    GPI_CUDA(&p, h2d(p, p.d_wav, wavptr.data(), wavptr.size() * sizeof(float *)));
    GPI_CUDA(&p, h2d(p, p.d_wav_ns, wavns.data(), wavns.size() * sizeof(int32_t)));
  }
  p.src_dirty = false;
  return GPI_OK;
}


int make_xcuts(int nx, int m, int npml, bool xlo, bool xhi, int *cuts) {
  const int E = 8;  // columns of an edge chunk
  // x-strip chunks: [E + 1, npml + 4) and [nx - npml - 5, nx - E), so that
  // the chunks between them meet no x strip (tile_class)
  const bool sl = xlo && npml + 4 > E + 1, sh = xhi && nx - npml - 5 < nx - E;
  const int lo = sl ? npml + 4 : E + 1, hi = sh ? nx - npml - 5 : nx - E;  // interior chunks cover [lo, hi)
  if (hi - lo < 2 * m || hi - lo < 16) {
    const int L = (nx + m - 1) / m;
    int n = 0;
    for (int x = 1; x <= nx; x += L) cuts[n++] = x;
    cuts[n] = nx + 1;
    return n;
  }
  // strip chunks no wider than the interior chunks (short column sweeps on
  // small grids)
  const int L = (hi - lo + m - 1) / m;
  auto split = [&](int a, int b, int *out) -> int {
    const int k = (b - a + L - 1) / L;
    for (int i = 0; i < k; i++) out[i] = a + (int)((int64_t)(b - a) * i / k);
    return k;
  };
  int n = 0;
  cuts[n++] = 1;
  if (sl) n += split(E + 1, lo, cuts + n);
  for (int i = 0; i < m; i++) cuts[n++] = lo + (int)((int64_t)(hi - lo) * i / m);
  if (sh) n += split(hi, nx - E, cuts + n);
  cuts[n++] = nx - E;  // the right edge chunk (hi itself without a right strip)
  cuts[n] = nx + 1;
  return n;
}

// Tile classes of the 2-D step kernels (src/fdtd/cpml.jl:184-211 and
// src/fdtd/dirichlet.jl:1-79 give the affected rows and columns):
//   0 interior: every cell it computes lies inside all update domains,
//     outside every CPML strip, away from mirror rows/columns and sources;
//   1 band: no x-edge or x-strip column; rows may meet a z strip, a z
//     mirror, the free surface or a source;
//   2 x-band: the same with x-strip columns;
//   3 edge: x-edge columns (domain ends and mirrors).
// A block computes velocities of rows z0..z0+TZ+2 and columns x0..x1+2 and
// stresses of rows z0..z0+TZ-1 and columns x0..x1-1 from input columns
// x0-3..x1+2.
static int tile_class(const Plan &p, const InjCell *cells, const int32_t *gptr, int zb, int x0, int x1, int shot) {
  const int npml = p.d.npml, nz = p.d.nz, nx = p.d.nx;
  const int z0 = 1 + zb * p.TZ;
  if (x0 <= 4 || x1 + 2 >= nx - 4) return 3;
  const bool xpml = p.d.pml_faces & (GPI_XMIN | GPI_XMAX);
  if (xpml && !(x0 > npml + 3 && x1 <= nx - 5 - npml)) return 2;
  for (int ipw = 0; ipw < p.d.npw; ipw++)
    for (int kind = 0; kind < NKIND; kind++) {
      const int gi = (ipw * p.d.nshots + shot) * NKIND + kind;
      for (int c = gptr[gi]; c < gptr[gi + 1]; c++)
        if (cells[c].col >= x0 - 3 && cells[c].col <= x1 + 3 && cells[c].row >= z0 - 1 &&
            cells[c].row <= z0 + p.TZ + 3)
          return 1;
    }
  const bool zin = z0 >= npml + 4 && z0 + p.TZ + 2 <= nz - npml - 3;
  return zin && x0 >= npml + 4 && x1 + 2 <= nx - npml - 3 ? 0 : 1;
}

int classify_tiles(const Plan &p, const int *xcut, const InjCell *cells, const int32_t *gptr, int4 *out, int cap,
                   int count[4]) {
  const int n = p.nzb * p.nxb * p.d.nshots;
  if (n > cap) return -1;
  int cnt[4] = {0, 0, 0, 0};
  for (int pass = 0; pass < 2; pass++) {
    int at[4] = {0, cnt[0], cnt[0] + cnt[1], cnt[0] + cnt[1] + cnt[2]};
    // shots innermost: the blocks of one (z-block, x-chunk) of every shot run
    // together and read the shared coefficient columns once from HBM, then
    // from L2
    for (int xb = 0; xb < p.nxb; xb++)
      for (int zb = 0; zb < p.nzb; zb++)
        for (int shot = 0; shot < p.d.nshots; shot++) {
          const int k = tile_class(p, cells, gptr, zb, xcut[xb], xcut[xb + 1], shot);
          if (pass == 0)
            cnt[k]++;
          else
            out[at[k]++] = make_int4(zb, xcut[xb], xcut[xb + 1], shot);
        }
  }
  for (int k = 0; k < 4; k++) count[k] = cnt[k];
  return n;
}

static int build_tiles(Plan &p) {
  const int n = p.nzb * p.nxb * p.d.nshots;
  std::vector<int4> t(n);
  const int32_t *gp = p.group_ptr.empty() ? nullptr : p.group_ptr.data();
  std::vector<int32_t> zero(2 * p.d.nshots * NKIND + 1, 0);
  if (classify_tiles(p, p.xcut.data(), p.h_cells.data(), gp ? gp : zero.data(), t.data(), n, p.n_tiles) < 0)
    return fail(&p, GPI_E_INVALID, "tile list");
  // injection cells per tile and class (the cells of a group are sorted by
  // column)
  const int32_t *g = gp ? gp : zero.data();
  const InjCell *cells = p.h_cells.data();
  for (auto &row : p.inj_tile)
    for (int &v : row) v = 0;
  for (int m = 0, at = 0; m < 4; m++)
    for (int i = 0; i < p.n_tiles[m]; i++, at++) {
      const int4 tl = t[at];
      int cw[2] = {0, 0};
      for (int ipw = 0; ipw < p.d.npw && ipw < 2; ipw++)
        for (int kind = 0; kind < NKIND; kind++) {
          const int gi = (ipw * p.d.nshots + tl.w) * NKIND + kind;
          const InjCell *b = cells + g[gi], *e = cells + g[gi + 1];
          const InjCell *lo = std::lower_bound(b, e, tl.y, [](const InjCell &c, int x) { return c.col < x; });
          const InjCell *hi = std::lower_bound(lo, e, tl.z + 3, [](const InjCell &c, int x) { return c.col < x; });
          cw[ipw] += (int)(hi - lo);
        }
      p.inj_tile[0][m] = std::max(p.inj_tile[0][m], cw[0]);
      p.inj_tile[1][m] = std::max(p.inj_tile[1][m], cw[1]);
      p.inj_tile[2][m] = std::max(p.inj_tile[2][m], cw[0] + cw[1]);
    }
  if (p.d_tiles) cudaFreeAsync(p.d_tiles, p.stream);
  p.d_tiles = nullptr;
  GPI_CUDA(&p, dalloc(p, (void **)&p.d_tiles, n * sizeof(int4)));
  GPI_CUDA(&p, h2d(p, p.d_tiles, t.data(), n * sizeof(int4)));
  p.h_tiles = t;
  return GPI_OK;
}

// ---------------------------------------------------------------------------
// run
// ---------------------------------------------------------------------------
static int step(Plan &p, int ipw_mask, int it, int mode, int vonly) {
  if (p.d.order != 4) return step_generic(&p, vonly);
  if (p.d.physics == GPI_ACOUSTIC)
    return p.d.ndim == 2 ? step_acoustic2d(&p, ipw_mask, it, mode, vonly) : step_acoustic3d(&p, ipw_mask, it, mode, vonly);
  return p.d.ndim == 2 ? step_elastic2d(&p, ipw_mask, it, mode, vonly) : step_elastic3d(&p, ipw_mask, it, mode, vonly);
}

static int zero_state(Plan &p) {
  for (int b = 0; b < 2; b++)
    for (int ipw = 0; ipw < p.d.npw; ipw++) {
      for (int f = 0; f < NFIELD; f++)
        if (p.state[b][ipw][f])
          GPI_CUDA(&p, cudaMemsetAsync(p.state[b][ipw][f], 0, p.fstride * p.d.nshots * sizeof(float), p.stream));
      for (int q = 0; q < p.nder; q++)
        if (p.psi[b][ipw][q])
          GPI_CUDA(&p, cudaMemsetAsync(p.psi[b][ipw][q], 0, p.psi_stride[q] * p.d.nshots * sizeof(float), p.stream));
    }
  p.cur[0] = p.cur[1] = 0;
  return GPI_OK;
}

static int run_body(Plan &p, int mode, bool chunked = false);

static bool same_sources(const std::vector<std::vector<Plan::Src>> &a, const std::vector<std::vector<Plan::Src>> &b) {
  if (a.size() != b.size()) return false;
  for (size_t s = 0; s < a.size(); s++) {
    if (a[s].size() != b[s].size()) return false;
    for (size_t f = 0; f < a[s].size(); f++) {
      const Plan::Src &x = a[s][f], &y = b[s][f];
      if (x.ns != y.ns || x.cp != y.cp || x.rv != y.rv || x.nz != y.nz || x.wav != y.wav) return false;
    }
  }
  return true;
}

void ckpt_prepare_forward(Plan *p);  // gpi_ckpt.cu

int run(Plan &p, int mode) {
  if (mode != GPI_FORWARD && mode != GPI_FORWARD_SAVE && mode != GPI_ADJOINT && mode != GPI_BORN)
    return fail(&p, GPI_E_INVALID, "mode");
  if (mode == GPI_BORN) {
    if (!p.have_born) return fail(&p, GPI_E_STATE, "Born run before gpi_set_born");
    for (auto &shot : p.src[1])
      for (auto &s : shot)
        if (s.ns) return fail(&p, GPI_E_STATE, "Born run: wavefield 2 takes no sources (clear them first)");
  }
  if (mode != GPI_FORWARD && p.d.npw != 2) return fail(&p, GPI_E_INVALID, "forward_save/adjoint need npw = 2");
  if (mode == GPI_ADJOINT && !p.have_save) return fail(&p, GPI_E_STATE, "adjoint run needs a forward_save run first");
  if (mode == GPI_ADJOINT && !((p.d.physics == GPI_ACOUSTIC && p.d.ndim == 2) || p.ck_slots > 0))
    return fail(&p, GPI_E_UNSUPPORTED,
                "gradients: 2-D acoustic media, or any checkpointed plan (the reference: 2-D acoustic)");
  if (mode == GPI_FORWARD_SAVE && p.d.physics == GPI_ELASTIC && p.ck_slots == 0)
    return fail(&p, GPI_E_UNSUPPORTED,
                "elastic gradients need a checkpointed plan (the reference defines no elastic gradient)");
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != p.device) GPI_CUDA(&p, cudaSetDevice(p.device));
  int rc = GPI_OK;
  // a checkpointed adjoint recomputes wavefield 1 with the sources of its
  // forward_save run, whatever the caller set for the time-reversed run
  // (update!(pa, srcwav, [-1, 1]) in gradient!, func_grad.jl:33)
  const bool swap_src = p.ck_slots > 0 && mode == GPI_ADJOINT && !same_sources(p.src[0], p.ck_src);
  if (swap_src) {
    std::swap(p.src[0], p.ck_src);
    p.src_dirty = true;
  }
  if (p.ck_slots > 0 && mode == GPI_FORWARD_SAVE) {
    ckpt_prepare_forward(&p);
    p.ck_src = p.src[0];
  }
  const bool recompile = p.rec_dirty || p.src_dirty || (p.d.ndim == 2 && !p.d_tiles);
  if (p.rec_dirty) rc = compile_receivers(p);
  if (!rc && p.src_dirty) {
    rc = compile_sources(p);
    if (!rc && p.d.ndim == 2) rc = build_tiles(p);
  }
  if (!rc && p.d.ndim == 2 && !p.d_tiles) rc = build_tiles(p);
  if (!rc && recompile) drop_graphs(p);
  if (!rc && mode == GPI_BORN) {
    // plain launches
    rc = zero_state(p);
    p.launches = 0;
    if (!rc && p.rec_pool)
      rc = cudaMemsetAsync(p.rec_pool, 0, p.rec_pool_floats * sizeof(float), p.stream) ? GPI_E_CUDA : 0;
    if (!rc) rc = born_coefficients(&p);
    if (!rc) rc = born_run(&p);
    if (!rc) {
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rc = fail(&p, GPI_E_CUDA, cudaGetErrorString(e));
    }
  } else if (!rc && p.graph_kind == 2) {
    rc = run_body(p, mode, true);
  } else if (!rc && p.graph_kind == 1) {
    // the whole run as one CUDA graph: captured on first use per mode,
    // replayed afterwards (the tables and buffers it uses keep their
    // addresses until the sources or receivers change)
    if (!p.gexec[mode]) {
      GPI_CUDA(&p, cudaStreamBeginCapture(p.stream, cudaStreamCaptureModeThreadLocal));
      rc = run_body(p, mode);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(p.stream, &graph);
      if (!rc && e != cudaSuccess) rc = fail(&p, GPI_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
      if (!rc && cudaGraphInstantiate(&p.gexec[mode], graph, 0) != cudaSuccess) {
        p.gexec[mode] = nullptr;
        rc = fail(&p, GPI_E_CUDA, "graph instantiation failed");
      }
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      p.glaunches[mode] = p.launches;
    }
    if (!rc) {
      GPI_CUDA(&p, cudaGraphLaunch(p.gexec[mode], p.stream));
      p.launches = p.glaunches[mode];
      if (mode == GPI_FORWARD_SAVE) p.have_save = 1;
    }
  } else if (!rc) {
    rc = run_body(p, mode);
  }
  if (swap_src) {
    std::swap(p.src[0], p.ck_src);
    p.src_dirty = true;
  }
  if (dev != p.device) cudaSetDevice(dev);
  return rc;
}

// A forward run split for a batch (gpi_batch.cu), which issues the steps of
// several plans together: what run() and run_body() do before the time loop
// (tables compiled, state and records zeroed) ...
int run_prepare_forward(Plan &p) {
  int rc = GPI_OK;
  const bool recompile = p.rec_dirty || p.src_dirty || !p.d_tiles;
  if (p.rec_dirty) rc = compile_receivers(p);
  if (!rc && p.src_dirty) {
    rc = compile_sources(p);
    if (!rc) rc = build_tiles(p);
  }
  if (!rc && !p.d_tiles) rc = build_tiles(p);
  if (!rc && recompile) drop_graphs(p);
  if (!rc) rc = zero_state(p);
  p.launches = 0;
  if (!rc && p.rec_pool)
    rc = cudaMemsetAsync(p.rec_pool, 0, p.rec_pool_floats * sizeof(float), p.stream) ? GPI_E_CUDA : 0;
  return rc;
}

// ... and after it: the velocity records of the last step and the extra
// velocity half step (propagate.jl:254-255)
int run_finish_forward(Plan &p) {
  int rc = aux_step(&p, p.d.nt + 1, GPI_FORWARD);
  if (!rc) rc = step(p, 1, p.d.nt + 1, GPI_FORWARD, 1);
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fail(&p, GPI_E_CUDA, cudaGetErrorString(e));
  }
  return rc;
}

int ensure_smem_attr(Plan *p, const void *fn, int slot, size_t bytes) {
  static std::mutex mu;
  static size_t done[32][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || slot < 0 || slot >= 32) return fail(p, GPI_E_UNSUPPORTED, "kernel slot or device index");
  std::lock_guard<std::mutex> lock(mu);
  if (done[slot][dev] >= bytes) return GPI_OK;
  GPI_CUDA(p, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  done[slot][dev] = bytes;
  return GPI_OK;
}

void drop_graphs(Plan &p) {
  for (int m = 0; m < 3; m++) {
    if (p.gexec[m]) cudaGraphExecDestroy(p.gexec[m]);
    p.gexec[m] = nullptr;
  }
  for (int m = 0; m < 3; m++) {
    if (p.cexec[m]) cudaGraphExecDestroy(p.cexec[m]);
    p.cexec[m] = nullptr;
  }
}


// the device work of one run: state reset, the time loop, the final half step
// one time step of the loop of mod_x_proc!; with `dev` its step index is
// the device counter plus `off` (inside a captured chunk)
// snaps_save! (src/fdtd/propagate.jl:238-245, src/fdtd/fdtd.jl:586-591):
// the snapshot field of every active wavefield after step it
static int save_snapshots(Plan &p, int mode, int it) {
  const int64_t n = p.fstride * p.d.nshots;
  const int npw = mode == GPI_ADJOINT ? 2 : 1;
  for (size_t k = 0; k < p.snap_its.size(); k++) {
    if (p.snap_its[k] != it) continue;
    for (int ipw = 0; ipw < npw; ipw++) {
      float *dst = p.snap_buf + ((int64_t)ipw * p.snap_its.size() + k) * n;
      GPI_CUDA(&p, cudaMemcpyAsync(dst, p.state[p.cur[ipw]][ipw][p.snap_field], n * sizeof(float),
                                   cudaMemcpyDeviceToDevice, p.stream));
    }
  }
  return GPI_OK;
}

static int step_body(Plan &p, int mode, int it, bool dev, int off) {
  const int mask = mode == GPI_ADJOINT ? 3 : 1;
  int rc = dev ? aux_step_dev(&p, off, mode) : aux_step(&p, it, mode);
  // boundary_force! (the replaced values are kept for the gradient)
  if (!rc && mode == GPI_ADJOINT) rc = dev ? boundary_io_dev(&p, off, 2) : boundary_io(&p, p.d.nt - it + 1, 2);
  if (!rc) rc = step(p, mask, it, mode, 0);
  if (!rc && mode == GPI_FORWARD_SAVE)
    rc = p.ck_slots > 0 ? ckpt_forward_store(&p, it) : dev ? boundary_io_dev(&p, off, 0) : boundary_io(&p, it, 0);
  if (!rc && !dev && p.snap_buf) rc = save_snapshots(p, mode, it);
  if (!rc && p.illum) rc = illum_add(&p);  // compute_illum! (propagate.jl:236)
  return rc;
}

// the steps [1, nchunks * K] as replays of one captured chunk of K steps
// (its aux and strip kernels read the step from the device counter, which
// the chunk advances at its end); returns the next plain step
static int run_chunks(Plan &p, int mode, int *next) {
  const int K = kChunkSteps, nchunks = p.d.nt / K;
  *next = 1;
  if (nchunks == 0) return GPI_OK;
  int rc = GPI_OK;
  if (!p.cexec[mode]) {
    const int64_t l0 = p.launches;
    const int c0 = p.cur[0], c1 = p.cur[1];
    GPI_CUDA(&p, cudaStreamBeginCapture(p.stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < K && !rc; k++) rc = step_body(p, mode, 0, true, k);
    if (!rc) rc = set_step(&p, K, 1);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(p.stream, &graph);
    if (!rc && e != cudaSuccess) rc = fail(&p, GPI_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    if (!rc && cudaGraphInstantiate(&p.cexec[mode], graph, 0) != cudaSuccess) {
      p.cexec[mode] = nullptr;
      rc = fail(&p, GPI_E_CUDA, "graph instantiation failed");
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    p.claunches[mode] = p.launches - l0;
    p.launches = l0;
    if (!rc && (p.cur[0] != c0 || p.cur[1] != c1)) rc = fail(&p, GPI_E_CUDA, "chunk does not end on its first buffers");
  }
  if (!rc) rc = set_step(&p, 1, 0);
  for (int c = 0; c < nchunks && !rc; c++) {
    if (cudaGraphLaunch(p.cexec[mode], p.stream) != cudaSuccess) rc = fail(&p, GPI_E_CUDA, "graph launch failed");
    p.launches += p.claunches[mode];
  }
  *next = nchunks * K + 1;
  return rc;
}

static int run_body(Plan &p, int mode, bool chunked) {
  if (mode == GPI_ADJOINT && p.ck_slots > 0) {
    p.launches = 0;
    int rc = ckpt_adjoint(&p);
    if (!rc) {
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rc = fail(&p, GPI_E_CUDA, cudaGetErrorString(e));
    }
    return rc;
  }
  int rc = zero_state(p);
  p.launches = 0;
  // initialize! (src/fdtd/types.jl:67-72): the illumination of this run
  if (!rc && p.illum)
    rc = cudaMemsetAsync(p.illum, 0, (size_t)p.fstride * p.d.nshots * sizeof(double), p.stream) ? GPI_E_CUDA : 0;
  // an adjoint run records nothing and keeps the records of the forward run
  if (!rc && p.rec_pool && mode != GPI_ADJOINT)
    rc = cudaMemsetAsync(p.rec_pool, 0, p.rec_pool_floats * sizeof(float), p.stream) ? GPI_E_CUDA : 0;
  if (!rc && mode == GPI_ADJOINT) {
    for (int i = 0; i < 3; i++)
      if (p.grad[i]) rc = cudaMemsetAsync(p.grad[i], 0, p.fstride * p.d.nshots * sizeof(float), p.stream) ? GPI_E_CUDA : rc;
    for (int i = 0; i < 2; i++)
      if (p.img[i]) rc = cudaMemsetAsync(p.img[i], 0, p.fstride * p.d.nshots * sizeof(float), p.stream) ? GPI_E_CUDA : rc;
    if (!rc) rc = snap_io(&p, 1, 1);
    if (!rc) rc = snap_io(&p, 0, 1);
  }
  int first = 1;
  // a checkpointed forward_save stores states and snapshots are taken at
  // host-chosen steps: plain
  if (!rc && chunked && !(mode == GPI_FORWARD_SAVE && p.ck_slots > 0) && !p.snap_buf) rc = run_chunks(p, mode, &first);
  for (int it = first; !rc && it <= p.d.nt; it++) rc = step_body(p, mode, it, false, 0);
  const bool snaps = mode == GPI_FORWARD_SAVE && p.ck_slots == 0;
  if (!rc) rc = aux_step(&p, p.d.nt + 1, mode);  // velocity records of the last step
  if (!rc && snaps) rc = snap_io(&p, 1, 0);
  if (!rc) rc = step(p, 1, p.d.nt + 1, mode, 1);  // the extra velocity half step (propagate.jl:254-255)
  if (!rc && snaps) rc = snap_io(&p, 0, 0);
  if (!rc && mode == GPI_ADJOINT && p.img[0]) rc = img_rho_finish(&p);
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fail(&p, GPI_E_CUDA, cudaGetErrorString(e));
  }
  if (!rc && mode == GPI_FORWARD_SAVE) p.have_save = 1;
  return rc;
}

// a kernel reports a pipeline wait that gave up through d_err
static int check_err(Plan &p) {
  int h = 0;
  GPI_CUDA(&p, cudaMemcpyAsync(&h, p.d_err, sizeof(int), cudaMemcpyDeviceToHost, p.stream));
  GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  if (h) {
    cudaMemsetAsync(p.d_err, 0, sizeof(int), p.stream);
    return fail(&p, GPI_E_CUDA, "a kernel's copy pipeline timed out; results of the last run are invalid");
  }
  return GPI_OK;
}

int transpose_records(Plan *p, float *out, const float *in, int nt, int nr);  // k_common.cu

int get_records(Plan &p, int shot, int field, float *out, int on_device) {
  if (shot < 0 || shot >= p.d.nshots || field < 0 || field >= NFIELD) return fail(&p, GPI_E_INVALID, "shot/field");
  const int nr = p.rec_n[shot][field];
  if (nr <= 0 || p.rec_base[shot][field] < 0) return fail(&p, GPI_E_STATE, "no receivers for this field (or no run yet)");
  const int nt = p.d.nt;
  const float *src = p.rec_pool + p.rec_base[shot][field];
  // pool layout [it][ir] -> Recs layout (it fastest)
  if (on_device) return transpose_records(&p, out, src, nt, nr);
  float *tmp = nullptr;
  GPI_CUDA(&p, pool_alloc((void **)&tmp, (size_t)nt * nr * sizeof(float), p.stream));
  int rc = transpose_records(&p, tmp, src, nt, nr);
  if (!rc) rc = cudaMemcpyAsync(out, tmp, (size_t)nt * nr * sizeof(float), cudaMemcpyDeviceToHost, p.stream)
                    ? fail(&p, GPI_E_CUDA, "records copy")
                    : GPI_OK;
  cudaFreeAsync(tmp, p.stream);
  if (rc) return rc;
  GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  return check_err(p);
}

int set_snapshots(Plan &p, int field, int n, const int *its) {
  if (p.snap_buf) cudaFreeAsync(p.snap_buf, p.stream);
  p.snap_buf = nullptr;
  p.snap_its.clear();
  p.snap_field = -1;
  if (field < 0 || n <= 0) return GPI_OK;
  if (field >= NFIELD || !p.present[field]) return fail(&p, GPI_E_INVALID, "snapshot field not in this physics");
  if (!its) return fail(&p, GPI_E_INVALID, "snapshot steps");
  for (int k = 0; k < n; k++)
    if (its[k] < 1 || its[k] > p.d.nt) return fail(&p, GPI_E_INVALID, "snapshot step outside 1..nt");
  p.snap_its.assign(its, its + n);
  p.snap_field = field;
  const size_t bytes = (size_t)p.d.npw * n * p.fstride * p.d.nshots * sizeof(float);
  if (pool_alloc((void **)&p.snap_buf, bytes, p.stream) != cudaSuccess) {
    cudaGetLastError();
    p.snap_buf = nullptr;
    p.snap_its.clear();
    return fail(&p, GPI_E_NOMEM, "snapshot buffer of " + std::to_string(bytes) + " bytes");
  }
  GPI_CUDA(&p, cudaMemsetAsync(p.snap_buf, 0, bytes, p.stream));
  drop_graphs(p);
  return GPI_OK;
}

int get_snapshot(Plan &p, int ipw, int k, int shot, float *out, int on_device) {
  if (!p.snap_buf) return fail(&p, GPI_E_STATE, "no snapshots configured");
  if (ipw < 1 || ipw > p.d.npw || k < 0 || k >= (int)p.snap_its.size() || shot < 0 || shot >= p.d.nshots)
    return fail(&p, GPI_E_INVALID, "ipw/snapshot/shot");
  int n[3];
  field_shape(p, p.snap_field, n);
  const float *src = p.snap_buf + (((int64_t)(ipw - 1) * p.snap_its.size() + k) * p.d.nshots + shot) * p.fstride;
  int rc = from_storage(p, out, src, n[0], n[1], n[2], on_device);
  if (rc) return rc;
  if (!on_device) {
    GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
    return check_err(p);
  }
  return GPI_OK;
}

// illum_flag (src/fdtd/fdtd.jl:59,177, types.jl:20): the per-shot sums of
// p^2 over the steps of each run (a checkpointed adjoint run keeps those of
// its forward_save run)
int set_illum(Plan &p, int enable) {
  if (enable && !p.present[GPI_P]) return fail(&p, GPI_E_UNSUPPORTED, "illumination sums p^2: acoustic media only");
  if (enable && p.d.nshots > 65535) return fail(&p, GPI_E_UNSUPPORTED, "illumination: at most 65535 shots per plan");
  if (!enable) {
    if (p.illum) cudaFreeAsync(p.illum, p.stream);
    p.illum = nullptr;
    drop_graphs(p);
    return GPI_OK;
  }
  if (p.illum) return GPI_OK;
  const size_t bytes = (size_t)p.fstride * p.d.nshots * sizeof(double);
  if (pool_alloc((void **)&p.illum, bytes, p.stream) != cudaSuccess) {
    cudaGetLastError();
    p.illum = nullptr;
    return fail(&p, GPI_E_NOMEM, "illumination buffer of " + std::to_string(bytes) + " bytes");
  }
  GPI_CUDA(&p, cudaMemsetAsync(p.illum, 0, bytes, p.stream));
  drop_graphs(p);
  return GPI_OK;
}

int get_illum(Plan &p, double *out, int on_device) {
  if (!p.illum) return fail(&p, GPI_E_STATE, "illumination not enabled");
  if (!out) return fail(&p, GPI_E_INVALID, "null argument");
  int64_t n = 1;
  {
    const int np = p.d.npml, f = p.d.pml_faces;
    const int lo[3] = {GPI_ZMIN, GPI_YMIN, GPI_XMIN}, hi[3] = {GPI_ZMAX, GPI_YMAX, GPI_XMAX};
    const int ext[3] = {p.d.nz, p.d.ndim == 3 ? p.d.ny : 1, p.d.nx};
    for (int a = 0; a < 3; a++)
      n *= (a == 1 && p.d.ndim == 2) ? 1 : ext[a] - ((f & lo[a]) ? np : 0) - ((f & hi[a]) ? np : 0);
  }
  if (on_device) return illum_stack(&p, out);
  double *tmp = nullptr;
  GPI_CUDA(&p, pool_alloc((void **)&tmp, (size_t)n * sizeof(double), p.stream));
  int rc = illum_stack(&p, tmp);
  if (!rc && cudaMemcpyAsync(out, tmp, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, p.stream))
    rc = fail(&p, GPI_E_CUDA, "illumination copy");
  cudaFreeAsync(tmp, p.stream);
  if (rc) return rc;
  GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  return check_err(p);
}

int get_field(Plan &p, int ipw, int shot, int field, float *out, int on_device) {
  if (ipw < 1 || ipw > p.d.npw || shot < 0 || shot >= p.d.nshots || field < 0 || field >= NFIELD || !p.present[field])
    return fail(&p, GPI_E_INVALID, "ipw/shot/field");
  int n[3];
  field_shape(p, field, n);
  const float *src = p.state[p.cur[ipw - 1]][ipw - 1][field] + p.fstride * shot;
  int rc = from_storage(p, out, src, n[0], n[1], n[2], on_device);
  if (rc) return rc;
  if (!on_device) {
    GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
    return check_err(p);
  }
  return GPI_OK;
}

int reduce_gradient(Plan *p, int param, float *dst);  // k_common.cu

int get_gradient(Plan &p, int param, float *out, int on_device) {
  if (p.d.npw != 2 || param < 0 || param >= p.nmod || !p.grad[param])
    return fail(&p, GPI_E_INVALID, "no gradient for this parameter");
  // sum over shots into shot 0's slot of a scratch area: reuse bstore's
  // snapshot region is not allowed (it is state), so reduce in place into a
  // temporary owned by the plan
  float *tmp = nullptr;
  GPI_CUDA(&p, pool_alloc((void **)&tmp, p.fstride * sizeof(float), p.stream));
  int rc = reduce_gradient(&p, param, tmp);
  if (!rc) rc = from_storage(p, out, tmp, p.d.nz, p.d.ny, p.d.nx, on_device);
  cudaFreeAsync(tmp, p.stream);
  if (rc) return rc;
  GPI_CUDA(&p, cudaStreamSynchronize(p.stream));
  return GPI_OK;
}

}  // namespace gpi

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace gpi;

extern "C" {

int gpi_plan_create(const gpi_plan_desc *desc, gpi_plan **out) { return gpi::create(desc, out); }
int gpi_plan_estimate(const gpi_plan_desc *desc, size_t *bytes) {
  if (!bytes) return gpi::fail(nullptr, GPI_E_INVALID, "null argument");
  return gpi::create(desc, nullptr, bytes);
}
void gpi_plan_destroy(gpi_plan *plan) { gpi::destroy(plan); }
const char *gpi_last_error(const gpi_plan *plan) { return plan ? plan->p.err.c_str() : g_create_err.c_str(); }
int gpi_set_stream(gpi_plan *plan, void *stream) {
  if (!plan) return GPI_E_INVALID;
  plan->p.stream = (cudaStream_t)stream;
  if (!stream && plan->p.use_graph) plan->p.stream = plan->p.own_stream;
  return GPI_OK;
}
int gpi_plan_bytes(const gpi_plan *plan, size_t *bytes) {
  if (!plan || !bytes) return GPI_E_INVALID;
  *bytes = plan->p.pool_bytes;
  return GPI_OK;
}
int gpi_set_medium(gpi_plan *plan, const float *const *mod, int on_device) {
  return plan ? gpi::set_medium(plan->p, mod, on_device) : GPI_E_INVALID;
}
int gpi_set_born(gpi_plan *plan, const float *const *dmod, int on_device) {
  return plan ? gpi::set_born(plan->p, dmod, on_device) : GPI_E_INVALID;
}
int gpi_set_pml(gpi_plan *plan, int q, int len, const float *a, const float *b, const float *kI) {
  return plan ? gpi::set_pml(plan->p, q, len, a, b, kI) : GPI_E_INVALID;
}
int gpi_set_sources(gpi_plan *plan, int ipw, int shot, int field, int ns, const int64_t *colptr, const int64_t *rowval,
                    const float *nzval, const float *wavelets) {
  return plan ? gpi::set_sources(plan->p, ipw, shot, field, ns, colptr, rowval, nzval, wavelets) : GPI_E_INVALID;
}
int gpi_clear_sources(gpi_plan *plan, int ipw, int shot) { return plan ? gpi::clear_sources(plan->p, ipw, shot) : GPI_E_INVALID; }
int gpi_set_adjoint_l2(gpi_plan *plan, int shot, int field, const float *dobs, int on_device, double *misfit) {
  return plan ? gpi::set_adjoint_l2(plan->p, shot, field, dobs, on_device, misfit) : GPI_E_INVALID;
}
int gpi_set_receivers(gpi_plan *plan, int shot, int field, int nr, const int64_t *colptr, const int64_t *rowval,
                      const float *nzval) {
  return plan ? gpi::set_receivers(plan->p, shot, field, nr, colptr, rowval, nzval) : GPI_E_INVALID;
}
int gpi_run(gpi_plan *plan, int mode) { return plan ? gpi::run(plan->p, mode) : GPI_E_INVALID; }
int gpi_get_records(gpi_plan *plan, int shot, int field, float *out, int on_device) {
  return plan ? gpi::get_records(plan->p, shot, field, out, on_device) : GPI_E_INVALID;
}
int gpi_get_gradient(gpi_plan *plan, int param, float *out, int on_device) {
  return plan ? gpi::get_gradient(plan->p, param, out, on_device) : GPI_E_INVALID;
}
int gpi_set_illum(gpi_plan *plan, int enable) { return plan ? gpi::set_illum(plan->p, enable) : GPI_E_INVALID; }
int gpi_get_illum(gpi_plan *plan, double *out, int on_device) {
  return plan ? gpi::get_illum(plan->p, out, on_device) : GPI_E_INVALID;
}
int gpi_set_snapshots(gpi_plan *plan, int field, int n, const int *its) {
  return plan ? gpi::set_snapshots(plan->p, field, n, its) : GPI_E_INVALID;
}
int gpi_get_snapshot(gpi_plan *plan, int ipw, int k, int shot, float *out, int on_device) {
  return plan ? gpi::get_snapshot(plan->p, ipw, k, shot, out, on_device) : GPI_E_INVALID;
}
int gpi_get_field(gpi_plan *plan, int ipw, int shot, int field, float *out, int on_device) {
  return plan ? gpi::get_field(plan->p, ipw, shot, field, out, on_device) : GPI_E_INVALID;
}
int gpi_set_graph(gpi_plan *plan, int enable) {
  if (!plan) return GPI_E_INVALID;
  // a graph cannot be captured on the legacy default stream: give the plan
  // a stream of its own
  if (enable && !plan->p.stream) {
    GPI_CUDA(&plan->p, cudaStreamCreateWithFlags(&plan->p.own_stream, cudaStreamNonBlocking));
    plan->p.stream = plan->p.own_stream;
  }
  if (enable < 0 || enable > 2) return GPI_E_INVALID;
  if (enable != plan->p.graph_kind) gpi::drop_graphs(plan->p);
  plan->p.use_graph = enable != 0;
  plan->p.graph_kind = enable;
  return GPI_OK;
}
int gpi_query(gpi_plan *plan, int *done) {
  if (!plan || !done) return GPI_E_INVALID;
  const cudaError_t e = cudaStreamQuery(plan->p.stream);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return GPI_OK;
  }
  *done = 1;
  return e == cudaSuccess ? GPI_OK : gpi::fail(&plan->p, GPI_E_CUDA, cudaGetErrorString(e));
}
int gpi_last_launches(const gpi_plan *plan, int64_t *launches) {
  if (!plan || !launches) return GPI_E_INVALID;
  *launches = plan->p.launches;
  return GPI_OK;
}

}  // extern "C"
