// k_common.cu -- small kernels shared by every physics:
//   * update coefficients from the medium (update_dmod!, src/fdtd/medium.jl:143-221)
//   * per-step auxiliary work: receiver gathers (record!, src/fdtd/receiver.jl:3-15)
//     and source amounts (mul!(pv, ssprayw, w) + muladd_*, src/fdtd/source.jl:61-177)
//   * boundary store for time reversal (src/fdtd/boundary.jl:1-306)
//   * shot-sum of gradients (sum_grads!, src/fdtd/gradient.jl:2-14)
//   * record transposition to the Recs layout (src/fdtd/receiver.jl:17-46)
// All arithmetic keeps the reference's operation order; the library is built
// without FMA contraction so that every product and sum rounds as written.
#include "gpi_internal.cuh"

namespace gpi {

struct Geo {
  int nz, ny, nx, NZP, NYP, ndim, h;
  __device__ __forceinline__ int64_t off(int r, int y, int c) const {
    return ((int64_t)(c - 1 + XOFF) * NYP + (ndim == 3 ? (y - 1 + YOFF) : 0)) * NZP + (r - 1 + ZOFF);
  }
};
static Geo geo(const Plan &p) { return Geo{p.d.nz, p.d.ny, p.d.nx, p.NZP, p.NYP, p.d.ndim, p.h}; }

// ---------------------------------------------------------------------------
// coefficients: each is stored at the cell it multiplies
// ---------------------------------------------------------------------------
struct CoefArgs {
  Geo g;
  float dt;
  int physics;
  const float *mod[3];
  float *coef[8];
};

__device__ __forceinline__ float invav2(float a, float b, float dt) { return dt / ((a + b) * 0.5f); }

__global__ void k_coef(CoefArgs a) {
  const Geo &g = a.g;
  const int h = g.h;
  const int64_t n1 = g.nz + h, n2 = g.ndim == 3 ? g.ny + h : 1, n3 = g.nx + h;
  const int64_t total = n1 * n2 * n3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i % n1) + 1;
    const int y = (int)((i / n1) % n2) + 1;
    const int c = (int)(i / (n1 * n2)) + 1;
    const int64_t o = g.off(r, y, c);
    const bool three = g.ndim == 3;
    const float *rho = a.mod[a.physics == GPI_ACOUSTIC ? 1 : 2];
    const bool yin = !three || (y >= h + 1 && y <= g.ny - h);
    // dtinvav{x}irho at the vx cell (r, y, c): rho[r, y, c-h], rho[r, y, c-h+1]
    if (r >= h + 1 && r <= g.nz - h && yin && c >= h + 1 && c <= g.nx)
      a.coef[0][o] = invav2(rho[g.off(r, y, c - h)], rho[g.off(r, y, c - h + 1)], a.dt);
    // dtinvav{z}irho at the vz cell (r, y, c): rho[r-h, y, c], rho[r-h+1, y, c]
    const int iz = three ? 2 : 1;
    if (r >= h + 1 && r <= g.nz && yin && c >= h + 1 && c <= g.nx - h)
      a.coef[iz][o] = invav2(rho[g.off(r - h, y, c)], rho[g.off(r - h + 1, y, c)], a.dt);
    // dtinvav{y}irho at the vy cell (r, y, c): rho[r, y-h, c], rho[r, y-h+1, c]
    if (three && r >= h + 1 && r <= g.nz - h && y >= h + 1 && y <= g.ny && c >= h + 1 && c <= g.nx - h)
      a.coef[1][o] = invav2(rho[g.off(r, y - h, c)], rho[g.off(r, y - h + 1, c)], a.dt);
    const bool full = r <= g.nz && y <= (three ? g.ny : 1) && c <= g.nx;
    if (a.physics == GPI_ACOUSTIC) {
      if (full) {
        const float t = 1.0f / a.mod[0][o];  // broadcast!(inv, dtK, invK)
        a.coef[three ? 3 : 2][o] = t * a.dt; // rmul!(dtK, dt)
      }
      continue;
    }
    const float *im = a.mod[1];
    if (full) {
      const float il = a.mod[0][o];
      const float lam = 1.0f / il;
      a.coef[three ? 7 : 4][o] = lam * a.dt;
      // inv(invλ) + 2.0 * inv(invμ) runs in Float64 (Float64 literal)
      const double m64 = (double)lam + 2.0 * (double)(1.0f / im[o]);
      a.coef[three ? 6 : 3][o] = (float)m64 * a.dt;
    }
    if (!three) {
      // dtavmu at the tauxz cell: dt / @av(invmu)
      if (r <= g.nz - h && c <= g.nx - h)
        a.coef[2][o] = a.dt / ((im[g.off(r, 1, c)] + im[g.off(r + 1, 1, c)] + im[g.off(r, 1, c + 1)] +
                                im[g.off(r + 1, 1, c + 1)]) * 0.25f);
    } else {
      // dtavxzimu at the tauxz cell (nz-h, ny-2h, nx-h): @av_xzi
      if (r <= g.nz - h && y <= g.ny - 2 * h && c <= g.nx - h)
        a.coef[3][o] = a.dt / ((im[g.off(r, y + h, c)] + im[g.off(r + 1, y + h, c)] + im[g.off(r, y + h, c + 1)] +
                                im[g.off(r + 1, y + h, c + 1)]) * 0.25f);
      // dtavxyimu at the tauxy cell (nz-2h, ny-h, nx-h): @av_xyi
      if (r <= g.nz - 2 * h && y <= g.ny - h && c <= g.nx - h)
        a.coef[4][o] = a.dt / ((im[g.off(r + h, y, c)] + im[g.off(r + h, y + 1, c)] + im[g.off(r + h, y, c + 1)] +
                                im[g.off(r + h, y + 1, c + 1)]) * 0.25f);
      // dtavyzimu at the tauyz cell (nz-h, ny-h, nx-2h): @av_yzi
      if (r <= g.nz - h && y <= g.ny - h && c <= g.nx - 2 * h)
        a.coef[5][o] = a.dt / ((im[g.off(r, y, c + h)] + im[g.off(r + 1, y, c + h)] + im[g.off(r, y + 1, c + h)] +
                                im[g.off(r + 1, y + 1, c + h)]) * 0.25f);
    }
  }
}

int compute_coefficients(Plan *p) {
  CoefArgs a;
  a.g = geo(*p);
  a.dt = (float)p->d.dt;
  a.physics = p->d.physics;
  for (int i = 0; i < 3; i++) a.mod[i] = p->mod[i];
  for (int i = 0; i < 8; i++) a.coef[i] = p->coef[i];
  for (int i = 0; i < p->ncoef; i++) GPI_CUDA(p, cudaMemsetAsync(p->coef[i], 0, p->fstride * sizeof(float), p->stream));
  k_coef<<<152 * 8, 256, 0, p->stream>>>(a);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// ---------------------------------------------------------------------------
// per-step auxiliary kernel
// ---------------------------------------------------------------------------
struct AuxArgs {
  const RecTask *tasks;
  int ntask;
  const int64_t *roff;
  const float *rw;
  float *rec;
  int it, nt;
  int it2, split;  // cells from `split` on (the adjoint wavefield's) take step it2
  int zero;        // write 0 for cells whose step is out of range
  const int *it_dev;  // when set: the step is *it_dev + it_off (graph-replayed step chunks)
  int it_off;
  const float *field[NFIELD];  // wavefield 1, current buffer, shot 0
  int64_t fs;
  const InjCell *cells;
  int ncells;
  const int32_t *pj;
  const float *pw;
  float *const *wav;
  float *amount;
  const float *rho;
  const float *kcoef;  // dtK or dtM
  float dt;
};

// thread i of one plan's aux work (records first, then injection cells);
// it, it2: the steps
__device__ __forceinline__ void aux_body(const AuxArgs &a, int i, int it, int it2) {
  if (i < a.ntask) {
    // record!: p is sampled before step it, velocities after step it-1
    const RecTask t = a.tasks[i];
    const bool isv = t.field == GPI_VX || t.field == GPI_VY || t.field == GPI_VZ;
    // the reference records p (before the step) and velocities (after the
    // velocity sources) only; other rfields keep their zero records
    if (!isv && t.field != GPI_P) return;
    const int tidx = isv ? it - 2 : it - 1;
    if (tidx < 0 || tidx >= a.nt) return;
    if (!isv && it > a.nt) return;
    const float *f = a.field[t.field] + t.shot * a.fs;
    float s = 0.f;
    for (int e = t.e0; e < t.e1; e++) s = s + a.rw[e] * f[a.roff[e]];
    a.rec[t.out + (int64_t)tidx * t.stride] = s;
    return;
  }
  i -= a.ntask;
  if (i >= a.ncells) return;
  const int itc = i < a.split ? it : it2;
  if (itc < 1 || itc > a.nt) {
    if (a.zero) a.amount[i] = 0.f;
    return;
  }
  const InjCell c = a.cells[i];
  const float *w = a.wav[c.wav] + (itc - 1);
  float pv = 0.f;
  for (int e = c.e0; e < c.e1; e++) pv = pv + a.pw[e] * w[(int64_t)a.pj[e] * a.nt];
  float amt;
  if (c.kind < 3)
    amt = pv / ((a.rho[c.roff0] + a.rho[c.roff1]) * 0.5f) * a.dt;  // muladd_with_density_v*!
  else
    amt = pv * a.kcoef[c.off];  // muladd_tauii!
  a.amount[i] = amt;
}

__global__ void k_aux(AuxArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (a.it_dev) {
    const int itd = *a.it_dev + a.it_off;
    aux_body(a, i, itd, itd);
  } else {
    aux_body(a, i, a.it, a.it2);
  }
}

// The aux work of several plans in one launch (a batch, gpi_batch.cu):
// plan k owns blocks [first[k], first[k+1]) and reads its arguments for
// this buffer parity (args[2 k + par]) and its step (*it_dev + off).
__global__ void k_aux_batch(const AuxArgs *__restrict__ args, const int *__restrict__ first, int nplans, int par,
                            int off) {
  __shared__ __align__(16) AuxArgs sa;
  __shared__ int s_k;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nplans - 1;  // the last plan whose first block is <= blockIdx.x
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (first[mid] <= (int)blockIdx.x)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_k = lo;
  }
  __syncthreads();
  const int k = s_k;
  const int *src = reinterpret_cast<const int *>(args + 2 * k + par);
  int *dst = reinterpret_cast<int *>(&sa);
  for (int j = threadIdx.x; j < (int)(sizeof(AuxArgs) / sizeof(int)); j += blockDim.x) dst[j] = src[j];
  __syncthreads();
  const int itd = *sa.it_dev + off;
  aux_body(sa, ((int)blockIdx.x - first[k]) * blockDim.x + threadIdx.x, itd, itd);
}

size_t aux_args_bytes() { return sizeof(AuxArgs); }

// a forward plan's aux arguments for both buffer parities (its step read
// from its device counter) and its block count (0: no aux work)
int aux_batch_args(Plan *p, void *out) {
  AuxArgs *o = static_cast<AuxArgs *>(out);
  const int n = p->n_rtask + p->n_cells;
  for (int par = 0; par < 2; par++) {
    AuxArgs &a = o[par];
    a = AuxArgs{};
    a.tasks = p->d_rtask;
    a.ntask = p->n_rtask;
    a.roff = p->d_roff;
    a.rw = p->d_rw;
    a.rec = p->rec_pool;
    a.it = a.it2 = 1;
    a.nt = p->d.nt;
    a.split = p->n_cells;
    a.zero = 0;
    a.it_dev = p->d_it;
    a.it_off = 0;
    for (int f = 0; f < NFIELD; f++) a.field[f] = p->state[p->cur[0] ^ par][0][f];
    a.fs = p->fstride;
    a.cells = p->d_cells;
    a.ncells = p->n_cells;
    a.pj = p->d_pair_j;
    a.pw = p->d_pair_w;
    a.wav = p->d_wav;
    a.amount = p->d_amount;
    a.rho = p->mod[p->d.physics == GPI_ACOUSTIC ? 1 : 2];
    a.kcoef = p->d.physics == GPI_ACOUSTIC ? p->coef[p->ncoef - 1] : p->coef[p->ncoef - 2];
    a.dt = (float)p->d.dt;
  }
  return (n + 127) / 128;
}

int aux_batch_launch(Plan *p, const void *args, const int *first, int nplans, int nblocks, int par, int off,
                     cudaStream_t st) {
  if (nblocks <= 0) return GPI_OK;
  k_aux_batch<<<nblocks, 128, 0, st>>>(static_cast<const AuxArgs *>(args), first, nplans, par, off);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// source amounts of wavefield 1 at step it1 and of the adjoint wavefield at
// step it2 (0: none), no records (the checkpointed adjoint)
int aux_step2(Plan *p, int it1, int it2) {
  if (!p->n_cells) return GPI_OK;
  AuxArgs a = {};
  a.ntask = 0;
  a.it = it1;
  a.it2 = it2;
  a.nt = p->d.nt;
  a.split = p->d.npw == 2 ? p->group_ptr[(size_t)p->d.nshots * NKIND] : p->n_cells;
  a.zero = 1;
  a.cells = p->d_cells;
  a.ncells = p->n_cells;
  a.pj = p->d_pair_j;
  a.pw = p->d_pair_w;
  a.wav = p->d_wav;
  a.amount = p->d_amount;
  a.rho = p->mod[p->d.physics == GPI_ACOUSTIC ? 1 : 2];
  a.kcoef = p->d.physics == GPI_ACOUSTIC ? p->coef[p->ncoef - 1] : p->coef[p->ncoef - 2];
  a.dt = (float)p->d.dt;
  k_aux<<<(p->n_cells + 127) / 128, 128, 0, p->stream>>>(a);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

int aux_step(Plan *p, int it, int mode) {
  // an adjoint run records nothing (get_update_parameters, propagate.jl:38-60)
  const int ntask = mode == GPI_ADJOINT ? 0 : p->n_rtask;
  const int n = ntask + (it <= p->d.nt ? p->n_cells : 0);
  if (n == 0) return GPI_OK;
  AuxArgs a;
  a.tasks = p->d_rtask;
  a.ntask = ntask;
  a.roff = p->d_roff;
  a.rw = p->d_rw;
  a.rec = p->rec_pool;
  a.it = it;
  a.nt = p->d.nt;
  a.it2 = it;
  a.split = p->n_cells;
  a.zero = 0;
  a.it_dev = nullptr;
  a.it_off = 0;
  // the records of a Born run are wavefield 2's
  const int rw = p->rec_ipw;
  for (int f = 0; f < NFIELD; f++) a.field[f] = p->state[p->cur[rw]][rw][f];
  a.fs = p->fstride;
  a.cells = p->d_cells;
  a.ncells = p->n_cells;
  a.pj = p->d_pair_j;
  a.pw = p->d_pair_w;
  a.wav = p->d_wav;
  a.amount = p->d_amount;
  a.rho = p->mod[p->d.physics == GPI_ACOUSTIC ? 1 : 2];
  a.kcoef = p->d.physics == GPI_ACOUSTIC ? p->coef[p->ncoef - 1] : p->coef[p->ncoef - 2];
  a.dt = (float)p->d.dt;
  k_aux<<<(n + 127) / 128, 128, 0, p->stream>>>(a);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// aux_step for step *d_it + off (the step chunks a CUDA graph replays)
int aux_step_dev(Plan *p, int off, int mode) {
  const int it = 1;  // cells are always launched; the kernel reads the step
  // an adjoint run records nothing (get_update_parameters, propagate.jl:38-60)
  const int ntask = mode == GPI_ADJOINT ? 0 : p->n_rtask;
  const int n = ntask + (it <= p->d.nt ? p->n_cells : 0);
  if (n == 0) return GPI_OK;
  AuxArgs a;
  a.tasks = p->d_rtask;
  a.ntask = ntask;
  a.roff = p->d_roff;
  a.rw = p->d_rw;
  a.rec = p->rec_pool;
  a.it = it;
  a.nt = p->d.nt;
  a.it2 = it;
  a.split = p->n_cells;
  a.zero = 0;
  a.it_dev = p->d_it;
  a.it_off = off;
  for (int f = 0; f < NFIELD; f++) a.field[f] = p->state[p->cur[0]][0][f];
  a.fs = p->fstride;
  a.cells = p->d_cells;
  a.ncells = p->n_cells;
  a.pj = p->d_pair_j;
  a.pw = p->d_pair_w;
  a.wav = p->d_wav;
  a.amount = p->d_amount;
  a.rho = p->mod[p->d.physics == GPI_ACOUSTIC ? 1 : 2];
  a.kcoef = p->d.physics == GPI_ACOUSTIC ? p->coef[p->ncoef - 1] : p->coef[p->ncoef - 2];
  a.dt = (float)p->d.dt;
  k_aux<<<(n + 127) / 128, 128, 0, p->stream>>>(a);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

__global__ void k_set_step(int *it, int v, int add) { *it = add ? *it + v : v; }

// the device step counter of the chunked runs: set (add = 0) or advance
int set_step(Plan *p, int v, int add) {
  k_set_step<<<1, 1, 0, p->stream>>>(p->d_it, v, add);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// ---------------------------------------------------------------------------
// boundary store (time reversal).  Per step and shot: for each saved stress
// field, the x strips (nz_f x 2nb), [the y strips,] the z strips (2nb x nx_f)
// of boundary_save! (boundary.jl:217-264); then the final snapshots.
// ---------------------------------------------------------------------------
struct StripArgs {
  Geo g;
  float *field;  // shot 0
  int64_t fs;
  float *store;  // shot 0, this step, this (field, axis) block
  int64_t sstride;  // floats per shot in the store
  int n1, n2, n3;   // field shape
  int axis, nb, np;
  int dir;          // 0 save (negated), 1 force, 2 force keeping the replaced values in prev
  int nshots;
  float *prev;      // dir 2: shot 0, this (field, axis) block, same layout and shot stride pstride
  int64_t pstride;
  // when set: the store block of step idx = *it_dev + it_off (dir 0) or
  // nt - (*it_dev + it_off) + 1 (dir 2), at store + (idx - 1) * bstep
  const int *it_dev;
  int it_off, nt;
  int64_t bstep;
};

__global__ void k_strip(StripArgs a) {
  const int b1 = a.axis == 0 ? 2 * a.nb : a.n1;
  const int b2 = a.axis == 1 ? 2 * a.nb : a.n2;
  const int b3 = a.axis == 2 ? 2 * a.nb : a.n3;
  const int64_t per = (int64_t)b1 * b2 * b3;
  const int64_t total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i % per;
    int i1 = (int)(k % b1), i2 = (int)((k / b1) % b2), i3 = (int)(k / ((int64_t)b1 * b2));
    int idx[3] = {i1, i2, i3};
    // strip entry j in [0, 2nb): j < nb -> np + j + 1 ; else n - np - nb + (j - nb) + 1
    const int j = idx[a.axis];
    const int nf = a.axis == 0 ? a.n1 : a.axis == 1 ? a.n2 : a.n3;
    const int fidx = j < a.nb ? a.np + j + 1 : nf - a.np - a.nb + (j - a.nb) + 1;
    int fi[3] = {i1 + 1, i2 + 1, i3 + 1};
    fi[a.axis] = fidx;
    float *f = a.field + shot * a.fs + a.g.off(fi[0], fi[1], fi[2]);
    float *s = a.store + shot * a.sstride + k;
    if (a.it_dev) {
      const int it = *a.it_dev + a.it_off;
      s += (int64_t)((a.dir == 0 ? it : a.nt - it + 1) - 1) * a.bstep;
    }
    if (a.dir == 0) {
      *s = -*f;
    } else {
      if (a.dir == 2) a.prev[shot * a.pstride + k] = *f;
      *f = *s;
    }
  }
}

static int saved_fields(const Plan &p, int *ids) {
  if (p.d.physics == GPI_ACOUSTIC) {
    ids[0] = GPI_P;
    return 1;
  }
  ids[0] = GPI_TAUXX;
  ids[1] = GPI_TAUXZ;
  ids[2] = GPI_TAUZZ;
  return 3;
}

static int boundary_impl(Plan *p, int it, int dir, bool dev, int off) {
  int ids[3];
  const int nsv = saved_fields(*p, ids);
  const int64_t sstride = p->bstep * p->d.nt + p->bsnap;
  float *st = p->bstore + (dev ? 0 : (int64_t)(it - 1) * p->bstep);
  float *pv = p->bprev;
  for (int q = 0; q < nsv; q++) {
    int kz, ky, kx;
    field_kinds(ids[q], &kz, &ky, &kx);
    const int n1 = nkind(kz, p->d.nz, p->h), n2 = p->d.ndim == 3 ? nkind(ky, p->d.ny, p->h) : 1,
              n3 = nkind(kx, p->d.nx, p->h);
    for (int axis = 2; axis >= 0; axis--) {
      if (axis == 1 && p->d.ndim == 2) continue;
      StripArgs a;
      a.g = geo(*p);
      a.field = p->state[p->cur[0]][0][ids[q]];
      a.fs = p->fstride;
      a.store = st;
      a.sstride = sstride;
      a.n1 = n1;
      a.n2 = n2;
      a.n3 = n3;
      a.axis = axis;
      a.nb = p->d.nbound;
      const int fmin = axis == 0 ? GPI_ZMIN : axis == 1 ? GPI_YMIN : GPI_XMIN;
      a.np = (p->d.pml_faces & fmin) ? p->d.npml : 0;
      a.dir = dir;
      a.nshots = p->d.nshots;
      a.prev = pv;
      a.pstride = p->bstep;
      a.it_dev = dev ? p->d_it : nullptr;
      a.it_off = off;
      a.nt = p->d.nt;
      a.bstep = p->bstep;
      int64_t per = 2 * (int64_t)p->d.nbound * (axis == 0 ? 1 : n1) * (axis == 1 ? 1 : n2) * (axis == 2 ? 1 : n3);
      int blocks = (int)std::min<int64_t>((per * p->d.nshots + 255) / 256, 152 * 16);
      k_strip<<<blocks, 256, 0, p->stream>>>(a);
      p->launches++;
      GPI_CUDA(p, cudaGetLastError());
      st += per;
      pv += per;
    }
  }
  return GPI_OK;
}

int boundary_io(Plan *p, int it, int dir) { return boundary_impl(p, it, dir, false, 0); }
int boundary_io_dev(Plan *p, int off, int dir) { return boundary_impl(p, 0, dir, true, off); }

// final snapshots: -tau (or -p) at nt and v after the extra half step, kept
// in storage layout after the strips of the last step
__global__ void k_snap(float *dst, const float *src, int64_t n, int64_t dstride, int64_t sstride, int nshots, int neg) {
  const int64_t total = n * nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(i / n);
    const int64_t k = i % n;
    const float v = src[s * sstride + k];
    dst[s * dstride + k] = neg ? -v : v;
  }
}

int snap_io(Plan *p, int tau, int dir) {
  int ids[3];
  const int nsv = saved_fields(*p, ids);
  const int64_t sstride = p->bstep * p->d.nt + p->bsnap;
  float *base = p->bstore + p->bstep * p->d.nt;
  const int vids[3] = {GPI_VX, GPI_VY, GPI_VZ};
  int slot = 0;
  auto one = [&](int f, int neg) -> int {
    float *snap = base + slot * p->fstride;
    float *fld = p->state[p->cur[0]][0][f];
    const int blocks = 152 * 8;
    if (dir == 0)
      k_snap<<<blocks, 256, 0, p->stream>>>(snap, fld, p->fstride, sstride, p->fstride, p->d.nshots, neg);
    else
      k_snap<<<blocks, 256, 0, p->stream>>>(fld, snap, p->fstride, p->fstride, sstride, p->d.nshots, 0);
    p->launches++;
    GPI_CUDA(p, cudaGetLastError());
    return GPI_OK;
  };
  for (int q = 0; q < nsv; q++, slot++)
    if (tau) {
      int rc = one(ids[q], 1);
      if (rc) return rc;
    }
  for (int q = 0; q < 3; q++) {
    if (q == 1 && p->d.ndim == 2) continue;
    if (!tau) {
      int rc = one(vids[q], 0);
      if (rc) return rc;
    }
    slot++;
  }
  return GPI_OK;
}

// ---------------------------------------------------------------------------
// gradient: sum over shots (the reference adds per-shot arrays on the host)
// ---------------------------------------------------------------------------
__global__ void k_shot_sum(float *dst, const float *src, int64_t n, int nshots) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < nshots; k++) s = s + src[k * n + i];
    dst[i] = s;
  }
}
int reduce_gradient(Plan *p, int param, float *dst) {
  k_shot_sum<<<152 * 8, 256, 0, p->stream>>>(dst, p->grad[param], p->fstride, p->d.nshots);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// compute_illum! (src/fdtd/fdtd.jl:571-582): illum[i] += abs2(p[i]), the
// square in FP32 and the sum in FP64, over the p cells of every shot
__global__ void k_illum(double *illum, const float *p, Geo g, int64_t fs) {
  const int r = blockIdx.y * 128 + threadIdx.x + 1;
  if (r > g.nz) return;
  const unsigned n2 = g.ndim == 3 ? g.ny : 1;
  const int y = (int)(blockIdx.x % n2) + 1, c = (int)(blockIdx.x / n2) + 1;
  const int64_t o = blockIdx.z * fs + g.off(r, y, c);
  const float v = p[o];
  illum[o] = illum[o] + (double)(v * v);
}
int illum_add(Plan *p) {
  const Geo g = geo(*p);
  const dim3 grid((unsigned)((p->d.ndim == 3 ? p->d.ny : 1) * p->d.nx), (p->d.nz + 127) / 128, p->d.nshots);
  k_illum<<<grid, 128, 0, p->stream>>>(p->illum, p->state[p->cur[0]][0][GPI_P], g, p->fstride);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// stack_illums! (src/fdtd/fdtd.jl:556-566): the sum over shots, in shot
// order from zero, of the cells of the physical grid (the padded faces
// dropped), column-major with z fastest
__global__ void k_illum_stack(double *dst, const double *illum, Geo g, int64_t fs, int nshots, int z0, int y0, int x0,
                              int mz, int my, int mx) {
  const int64_t n = (int64_t)mz * my * mx;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int iz = (int)(i % mz), iy = (int)((i / mz) % my), ix = (int)(i / ((int64_t)mz * my));
    const int64_t o = g.off(z0 + iz, y0 + iy, x0 + ix);
    double s = 0.0;
    for (int k = 0; k < nshots; k++) s = s + illum[k * fs + o];
    dst[i] = s;
  }
}
int illum_stack(Plan *p, double *dst) {
  const int np = p->d.npml;
  const int f = p->d.pml_faces;
  const int z0 = 1 + ((f & GPI_ZMIN) ? np : 0), mz = p->d.nz - ((f & GPI_ZMIN) ? np : 0) - ((f & GPI_ZMAX) ? np : 0);
  const int x0 = 1 + ((f & GPI_XMIN) ? np : 0), mx = p->d.nx - ((f & GPI_XMIN) ? np : 0) - ((f & GPI_XMAX) ? np : 0);
  int y0 = 1, my = 1;
  if (p->d.ndim == 3) {
    y0 = 1 + ((f & GPI_YMIN) ? np : 0);
    my = p->d.ny - ((f & GPI_YMIN) ? np : 0) - ((f & GPI_YMAX) ? np : 0);
  }
  k_illum_stack<<<152 * 4, 256, 0, p->stream>>>(dst, p->illum, geo(*p), p->fstride, p->d.nshots, z0, y0, x0, mz, my,
                                                mx);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// records: pool [it][ir] -> Recs layout [ir][it]
__global__ void k_transpose(float *out, const float *in, int nt, int nr) {
  __shared__ float tile[32][33];
  const int it0 = blockIdx.x * 32, ir0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int it = it0 + k, ir = ir0 + threadIdx.x;
    if (it < nt && ir < nr) tile[k][threadIdx.x] = in[(int64_t)it * nr + ir];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int ir = ir0 + k, it = it0 + threadIdx.x;
    if (it < nt && ir < nr) out[(int64_t)ir * nt + it] = tile[threadIdx.x][k];
  }
}
int transpose_records(Plan *p, float *out, const float *in, int nt, int nr) {
  dim3 grid((nt + 31) / 32, (nr + 31) / 32);
  k_transpose<<<grid, dim3(32, 8), 0, p->stream>>>(out, in, nt, nr);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// gradient!'s adjoint sources for L2DistLoss (src/fdtd/func_grad.jl:11-49)
// from the records in the pool ([it][ir]) and observed data dobs (Recs
// layout, [ir][it]): adj[ir][nt-1-it] = 2 (dobs - dcal) (deriv(loss, dobs,
// dcal), reverse!) and per block the sum of (dobs - dcal)^2 in double, each
// 32 x 32 tile transposed through shared memory and summed in a fixed order
__global__ void k_adjoint_l2(float *adj, double *partial, const float *dobs, const float *rec, int nt, int nr) {
  __shared__ float tile[32][33];
  __shared__ double red[256];
  const int it0 = blockIdx.x * 32, ir0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int it = it0 + k, ir = ir0 + threadIdx.x;
    if (it < nt && ir < nr) tile[k][threadIdx.x] = rec[(int64_t)it * nr + ir];
  }
  __syncthreads();
  double acc = 0.0;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int ir = ir0 + k, it = it0 + threadIdx.x;
    if (it < nt && ir < nr) {
      const float ob = dobs[(int64_t)ir * nt + it], dc = tile[threadIdx.x][k];
      adj[(int64_t)ir * nt + (nt - 1 - it)] = 2.0f * (ob - dc);
      const double e = (double)ob - (double)dc;
      acc += e * e;
    }
  }
  const int t = threadIdx.y * 32 + threadIdx.x;
  red[t] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) red[t] += red[t + w];
    __syncthreads();
  }
  if (t == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}
// the partial sums in order (one thread: a few thousand values)
__global__ void k_sum_ordered(double *out, const double *partial, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += partial[i];
  *out = s;
}
int adjoint_l2_launch(Plan *p, float *adj, double *partial, double *out, const float *dobs, const float *rec, int nt,
                      int nr) {
  dim3 grid((nt + 31) / 32, (nr + 31) / 32);
  k_adjoint_l2<<<grid, dim3(32, 8), 0, p->stream>>>(adj, partial, dobs, rec, nt, nr);
  k_sum_ordered<<<1, 1, 0, p->stream>>>(out, partial, (int)(grid.x * grid.y));
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}
int adjoint_l2_blocks(int nt, int nr) { return ((nt + 31) / 32) * ((nr + 31) / 32); }

}  // namespace gpi
