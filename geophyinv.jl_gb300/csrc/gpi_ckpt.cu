// gpi_ckpt.cu -- checkpointed adjoint: the gradient of gradient! without the
// boundary store.
//
// The reference rebuilds the forward wavefield backwards in time from strips
// saved at every step (boundary_save!/boundary_force!, src/fdtd/boundary.jl)
// and correlates it with the adjoint wavefield (compute_gradient!,
// src/fdtd/gradient.jl:27-56).  A checkpointed plan instead keeps a few
// full states of wavefield 1 (fields and CPML memory) in device slots during
// the forward_save run and, in the adjoint run, recomputes the forward states
// it needs from them on a binomial ("revolve") schedule (Griewank & Walther,
// ACM TOMS 26(1), 2000).  Memory: slots x one state, independent of nt, so
// 3-D gradients fit on the device.
//
// Adjoint step j reverses forward step s = nt - j + 1.  With P_k, V_k the
// forward pressure and velocities after step k (V_{nt+1} after the extra
// half step), the time-reversed run of the reference holds
//   before step j: p1 = -P_s,      v1 = V_{s+1}
//   after  step j: p1 = -P_{s-1},  v1 = V_s
// so its imaging condition is
//   g_invK += p2_prev (P_{s-1} - P_s) dtI
//   b_v     = v2_prev (V_s - V_{s+1}) dtI   (then combined into g_rho)
// A "turn" at s therefore starts from the full state s-1 in buffer A, runs
// forward step s into B (B = state s, A still holds P_{s-1}), runs the
// velocity half step of step s+1 (with its velocity sources; none after
// step nt, as the reference's extra half step) back into A's velocities
// without writing A's pressure, and calls the imaging kernel on (A, B) and
// the adjoint wavefield before it takes adjoint step j.  3-D steps update in
// place, so the old pressure and velocities are copied aside instead.
// Outside the reference's strips (3 cells at the PML edge) and the cells
// whose averages reach into the PML, the result equals the reference's
// gradient up to rounding; there the reference correlates with values the
// time-reversed run left unforced.
#include "k_stencil.cuh"

#include <algorithm>
#include <cmath>

namespace gpi {

// ---------------------------------------------------------------------------
// the schedule (host)
// ---------------------------------------------------------------------------
namespace {

// beta(c, r) = C(c + r, c): steps reversible with c checkpoints and at most
// r advances of any step (Griewank & Walther); 0 for r < 0
double beta(int c, int r) {
  if (r < 0) return 0.0;
  double b = 1.0;
  for (int i = 1; i <= c; i++) b = b * (double)(r + i) / (double)i;
  return std::floor(b + 0.5);
}

// fewest forward steps (turn steps not counted) that reverse l steps with c
// checkpoints, one of which holds the starting state
double rev_cost(int64_t l, int c) {
  if (l <= 1) return 0.0;
  if (c <= 1) return (double)l * (double)(l - 1) / 2.0;
  int r = 1;
  while (beta(c, r) < (double)l) r++;
  return (double)r * (double)l - beta(c + 1, r - 1);
}

int best_split(int n, int c) {
  int best = 1;
  double bc = 1e300;
  for (int m = 1; m < n; m++) {
    const double v = m + rev_cost(n - m, c - 1) + rev_cost(m, c);
    if (v < bc) {
      bc = v;
      best = m;
    }
  }
  return best;
}

enum { OP_RESTORE = 0, OP_ADVANCE = 1, OP_STORE = 2, OP_TURN = 3 };
struct Op {
  int kind, slot, a, b;  // restore: slot (-1 zero state), state a; advance: a -> b; store: slot, a; turn: step a
};
struct Sched {
  std::vector<Op> ops;
  std::vector<std::pair<int, int>> first;
  std::vector<int> free_slots;
  int64_t advances = 0, turns = 0;
};

void rev(Sched &S, int a, int aslot, int n, int c, bool first) {
  if (n <= 0) return;
  if (n == 1) {
    S.ops.push_back({OP_RESTORE, aslot, a, 0});
    S.ops.push_back({OP_TURN, -1, a + 1, 0});
    S.turns++;
    return;
  }
  if (c <= 1 || S.free_slots.empty()) {
    for (int k = n; k >= 1; k--) {
      S.ops.push_back({OP_RESTORE, aslot, a, 0});
      if (k > 1) {
        S.ops.push_back({OP_ADVANCE, -1, a, a + k - 1});
        S.advances += k - 1;
      }
      S.ops.push_back({OP_TURN, -1, a + k, 0});
      S.turns++;
    }
    return;
  }
  const int m = best_split(n, c);
  const int slot = S.free_slots.back();
  S.free_slots.pop_back();
  if (first) {
    S.first.push_back({a + m, slot});
  } else {
    S.ops.push_back({OP_RESTORE, aslot, a, 0});
    S.ops.push_back({OP_ADVANCE, -1, a, a + m});
    S.ops.push_back({OP_STORE, slot, a + m, 0});
    S.advances += m;
  }
  rev(S, a + m, slot, n - m, c - 1, first);
  S.free_slots.push_back(slot);
  rev(S, a, aslot, m, c, false);
}

Sched schedule(int nt, int slots) {
  Sched S;
  for (int i = slots - 1; i >= 0; i--) S.free_slots.push_back(i);
  // the zero initial state counts as a checkpoint that costs no slot
  rev(S, 0, -1, nt, slots + 1, true);
  return S;
}

}  // namespace

// ---------------------------------------------------------------------------
// slots: fields then CPML memory of wavefield 1, each 64-float aligned
// ---------------------------------------------------------------------------
template <class F>
static void for_state(const Plan &p, int buf, F &&fn) {
  int64_t off = 0;
  for (int f = 0; f < NFIELD; f++)
    if (p.present[f] && p.state[buf][0][f]) {
      const int64_t n = p.fstride * p.d.nshots;
      fn(p.state[buf][0][f], off, n);
      off += (n + 63) / 64 * 64;
    }
  for (int q = 0; q < p.nder; q++)
    if (p.psi[buf][0][q] && p.psi_stride[q] > 0) {
      const int64_t n = p.psi_stride[q] * p.d.nshots;
      fn(p.psi[buf][0][q], off, n);
      off += (n + 63) / 64 * 64;
    }
}

int64_t ckpt_slot_floats(const Plan &p) {
  int64_t total = 0;
  for (int f = 0; f < NFIELD; f++)
    if (p.present[f]) total += (p.fstride * p.d.nshots + 63) / 64 * 64;
  for (int q = 0; q < p.nder; q++)
    if (p.psi_stride[q] > 0) total += (p.psi_stride[q] * p.d.nshots + 63) / 64 * 64;
  return total;
}

static int slot_copy(Plan *p, int slot, bool store) {
  float *base = p->ck_pool + (int64_t)slot * p->ck_floats;
  const int buf = store ? p->cur[0] : 0;
  int rc = GPI_OK;
  for_state(*p, buf, [&](float *arr, int64_t off, int64_t n) {
    if (rc) return;
    const cudaError_t e = store ? cudaMemcpyAsync(base + off, arr, n * sizeof(float), cudaMemcpyDeviceToDevice, p->stream)
                                : cudaMemcpyAsync(arr, base + off, n * sizeof(float), cudaMemcpyDeviceToDevice, p->stream);
    if (e != cudaSuccess) rc = fail(p, GPI_E_CUDA, std::string("checkpoint copy: ") + cudaGetErrorString(e));
  });
  if (!store) p->cur[0] = 0;
  return rc;
}

static int zero_wavefield(Plan *p, int ipw) {
  for (int b = 0; b < 2; b++) {
    for (int f = 0; f < NFIELD; f++)
      if (p->state[b][ipw][f])
        GPI_CUDA(p, cudaMemsetAsync(p->state[b][ipw][f], 0, p->fstride * p->d.nshots * sizeof(float), p->stream));
    for (int q = 0; q < p->nder; q++)
      if (p->psi[b][ipw][q])
        GPI_CUDA(p, cudaMemsetAsync(p->psi[b][ipw][q], 0, p->psi_stride[q] * p->d.nshots * sizeof(float), p->stream));
  }
  p->cur[ipw] = 0;
  return GPI_OK;
}

int ckpt_forward_store(Plan *p, int it) {
  for (auto &fs : p->ck_first)
    if (fs.first == it) return slot_copy(p, fs.second, true);
  return GPI_OK;
}

// ---------------------------------------------------------------------------
// imaging condition, 3-D acoustic (the 2-D one is k_grad_a2): the 2-D
// formulas with a y term, g_rho - avx - avy - avz
// ---------------------------------------------------------------------------
struct Grad3Args {
  int nz, ny, nx, NZP, NYP;
  int64_t fs;
  int nshots;
  const float *p2, *pold, *pnew;
  const float *v2[3], *vs[3], *vs1[3];  // x, y, z: adjoint, V_s, V_{s+1}
  float *gK, *gR;
  float dtI;
  int imaging;  // 0 the reference-style rho term, 1 the discrete model's
};

__global__ void __launch_bounds__(256) k_grad_a3(const Grad3Args a) {
  const int64_t per = (int64_t)a.nz * a.ny * a.nx;
  const int64_t total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    int64_t k = i - shot * per;
    const int r = (int)(k % a.nz) + 1;
    k /= a.nz;
    const int y = (int)(k % a.ny) + 1, c = (int)(k / a.ny) + 1;
    const int64_t so = shot * a.fs;
    auto S = [&](int rr, int yy, int cc) -> int64_t {
      return so + ((int64_t)(cc - 1 + XOFF) * a.NYP + (yy - 1 + YOFF)) * a.NZP + (rr - 1 + ZOFF);
    };
    const int64_t o = S(r, y, c);
    a.gK[o] = a.gK[o] + a.p2[o] * (a.pold[o] - a.pnew[o]) * a.dtI;
    if (a.imaging) {
      // rho(r, y, c) sits in the coefficients of the velocity cells two and
      // three cells further along each axis, where those are updated (vx:
      // rows 4..nz-3, y 4..ny-3, columns 4..nx; vy: rows 4..nz-3, y 4..ny,
      // columns 4..nx-3; vz: rows 4..nz, y 4..ny-3, columns 4..nx-3)
      auto b = [&](int d, int rr, int yy, int cc, bool in) {
        const int64_t q = S(rr, yy, cc);
        return in ? a.v2[d][q] * (a.vs[d][q] - a.vs1[d][q]) * a.dtI : 0.f;
      };
      const bool rin = r >= 4 && r <= a.nz - 3, yin = y >= 4 && y <= a.ny - 3, cin = c >= 4 && c <= a.nx - 3;
      const float avx = rin && yin ? (b(0, r, y, c + 2, c + 2 >= 4 && c + 2 <= a.nx) +
                                      b(0, r, y, c + 3, c + 3 >= 4 && c + 3 <= a.nx)) * 0.5f : 0.f;
      const float avy = rin && cin ? (b(1, r, y + 2, c, y + 2 >= 4 && y + 2 <= a.ny) +
                                      b(1, r, y + 3, c, y + 3 >= 4 && y + 3 <= a.ny)) * 0.5f : 0.f;
      const float avz = yin && cin ? (b(2, r + 2, y, c, r + 2 >= 4 && r + 2 <= a.nz) +
                                      b(2, r + 3, y, c, r + 3 >= 4 && r + 3 <= a.nz)) * 0.5f : 0.f;
      a.gR[o] = a.gR[o] - avx - avy - avz;
    } else if (r >= 4 && r <= a.nz - 3 && y >= 4 && y <= a.ny - 3 && c >= 4 && c <= a.nx - 3) {
      auto b = [&](int d, int64_t q) { return a.v2[d][q] * (a.vs[d][q] - a.vs1[d][q]) * a.dtI; };
      const float bx1 = b(0, S(r, y, c - 3)), bx2 = b(0, S(r, y, c - 2));
      const float by1 = b(1, S(r, y - 3, c)), by2 = b(1, S(r, y - 2, c));
      const float bz1 = b(2, S(r - 3, y, c)), bz2 = b(2, S(r - 2, y, c));
      a.gR[o] = a.gR[o] - (bx1 + bx2) * 0.5f - (by1 + by2) * 0.5f - (bz1 + bz2) * 0.5f;
    }
  }
}

// ---------------------------------------------------------------------------
// imaging condition, 3-D elastic (no counterpart in the reference, which
// defines gradients for 2-D acoustic media only): the gradient of the
// discrete scheme with respect to invlambda, invmu and rho.  Per step, with
// X the forward state before step s, W after it (velocities: after the
// velocity half step of s+1) and Y the adjoint state before adjoint step j:
//   normal-stress cells: K = (dtM - dtl) I + dtl 1 1', a = K^-1 Y_n,
//     b = K^-1 (X_n - W_n);  g_invlambda += (sum a)(sum b) dtl^2 / dt,
//     g_invmu += (a . b) 2 dt / invmu^2
//   shear cells: a quarter of Y_s (X_s - W_s) / dt to each of the four
//     invmu cells of the cell's average (@av_xzi, @av_xyi, @av_yzi)
//   velocity cells: the rho term of the acoustic discrete-model imaging
//     condition (imaging = 1)
// (K^-1 turns a stress into the strain that produced it, so no derivative
// is recomputed.)  Checked against finite differences of the misfit.
// ---------------------------------------------------------------------------
struct GradE3Args {
  int nz, ny, nx, NZP, NYP;
  int64_t fs;
  int nshots;
  const float *Y[NFIELD], *X[NFIELD], *W[NFIELD];
  const float *dtM, *dtl, *invmu;
  float *gL, *gM, *gR;
  float dt, dtI;
};

__global__ void __launch_bounds__(256) k_grad_e3(const GradE3Args a) {
  const int64_t per = (int64_t)a.nz * a.ny * a.nx;
  const int64_t total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    int64_t k = i - shot * per;
    const int r = (int)(k % a.nz) + 1;
    k /= a.nz;
    const int y = (int)(k % a.ny) + 1, c = (int)(k / a.ny) + 1;
    const int64_t so = shot * a.fs;
    auto L = [&](int rr, int yy, int cc) -> int64_t {
      return ((int64_t)(cc - 1 + XOFF) * a.NYP + (yy - 1 + YOFF)) * a.NZP + (rr - 1 + ZOFF);
    };
    const int64_t lo = L(r, y, c), o = so + lo;
    // normal stresses
    const int nid[3] = {GPI_TAUXX, GPI_TAUYY, GPI_TAUZZ};
    float q[3], dT[3], sq = 0.f, sT = 0.f;
#pragma unroll
    for (int m = 0; m < 3; m++) {
      q[m] = a.Y[nid[m]][o];
      dT[m] = a.X[nid[m]][o] - a.W[nid[m]][o];
      sq = sq + q[m];
      sT = sT + dT[m];
    }
    const float beta = a.dtl[lo], alpha = a.dtM[lo] - a.dtl[lo];
    const float cq = beta / (alpha + 3.0f * beta);
    float sa = 0.f, sb = 0.f, ab = 0.f;
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const float am = (q[m] - cq * sq) / alpha, bm = (dT[m] - cq * sT) / alpha;
      sa = sa + am;
      sb = sb + bm;
      ab = ab + am * bm;
    }
    const float im = a.invmu[lo];
    a.gL[o] = a.gL[o] + sa * sb * (beta * beta * a.dtI);
    float gm = a.gM[o] + ab * (2.0f * a.dt / (im * im));
    // shear stresses whose invmu average holds this cell, in the order
    // tauxz, tauxy, tauyz and, within each, by column, y, row
    auto sh = [&](int f, int rr, int yy, int cc) -> float {
      const int64_t s = so + L(rr, yy, cc);
      return a.Y[f][s] * (a.X[f][s] - a.W[f][s]) * a.dtI * 0.25f;
    };
    const int nz = a.nz, ny = a.ny, nx = a.nx;
    // tauxz (nz-3, ny-6, nx-3): cell (iz, iy, ix) averages rows iz, iz+1,
    // y iy+3, columns ix, ix+1
    if (y - 3 >= 1 && y - 3 <= ny - 6)
      for (int cc = c - 1; cc <= c; cc++)
        for (int rr = r - 1; rr <= r; rr++)
          if (cc >= 1 && cc <= nx - 3 && rr >= 1 && rr <= nz - 3) gm = gm + sh(GPI_TAUXZ, rr, y - 3, cc);
    // tauxy (nz-6, ny-3, nx-3): row iz+3, y iy, iy+1, columns ix, ix+1
    if (r - 3 >= 1 && r - 3 <= nz - 6)
      for (int cc = c - 1; cc <= c; cc++)
        for (int yy = y - 1; yy <= y; yy++)
          if (cc >= 1 && cc <= nx - 3 && yy >= 1 && yy <= ny - 3) gm = gm + sh(GPI_TAUXY, r - 3, yy, cc);
    // tauyz (nz-3, ny-3, nx-6): rows iz, iz+1, y iy, iy+1, column ix+3
    if (c - 3 >= 1 && c - 3 <= nx - 6)
      for (int yy = y - 1; yy <= y; yy++)
        for (int rr = r - 1; rr <= r; rr++)
          if (yy >= 1 && yy <= ny - 3 && rr >= 1 && rr <= nz - 3) gm = gm + sh(GPI_TAUYZ, rr, yy, c - 3);
    a.gM[o] = gm;
    // rho: velocity cells two and three cells further along each axis
    auto b = [&](int f, int rr, int yy, int cc, bool in) -> float {
      const int64_t s = so + L(rr, yy, cc);
      return in ? a.Y[f][s] * (a.X[f][s] - a.W[f][s]) * a.dtI : 0.f;  // V_s - V_{s+1}
    };
    const bool rin = r >= 4 && r <= nz - 3, yin = y >= 4 && y <= ny - 3, cin = c >= 4 && c <= nx - 3;
    const float avx = rin && yin ? (b(GPI_VX, r, y, c + 2, c + 2 >= 4 && c + 2 <= nx) +
                                    b(GPI_VX, r, y, c + 3, c + 3 >= 4 && c + 3 <= nx)) * 0.5f : 0.f;
    const float avy = rin && cin ? (b(GPI_VY, r, y + 2, c, y + 2 >= 4 && y + 2 <= ny) +
                                    b(GPI_VY, r, y + 3, c, y + 3 >= 4 && y + 3 <= ny)) * 0.5f : 0.f;
    const float avz = yin && cin ? (b(GPI_VZ, r + 2, y, c, r + 2 >= 4 && r + 2 <= nz) +
                                    b(GPI_VZ, r + 3, y, c, r + 3 >= 4 && r + 3 <= nz)) * 0.5f : 0.f;
    a.gR[o] = a.gR[o] - avx - avy - avz;
  }
}

// The source terms at the cells of explosive sources (stress kind): the
// forward step added A = dtM pv to every normal stress there, so the stress
// decrease is K e - A 1 and dtM also multiplies the source; with
// sa = sum(K^-1 q) and corr = A / (dtM + 2 dtl):
//   g_invlambda += sa (3 corr - A / dtM) dtl^2 / dt
//   g_invmu     += sa (corr - A / dtM) 2 dt / invmu^2
// added right after forward step s (while the cells' amounts are those of
// step s), before the main kernel's terms.  One thread per shot walks its
// cells in order (two source fields may share a cell).
struct GradE3SrcArgs {
  int64_t fs;
  int nshots;
  const InjCell *cells;
  const int32_t *gptr;  // wavefield 1's groups
  const float *amount;
  const float *Y[3], *dtM, *dtl, *invmu;  // Y: adjoint txx, tyy, tzz
  float *gL, *gM;
  float dt, dtI;
};

__global__ void k_grad_e3_src(const GradE3SrcArgs a) {
  const int shot = blockIdx.x * blockDim.x + threadIdx.x;
  if (shot >= a.nshots) return;
  const int g = shot * NKIND + 3;
  const int64_t so = shot * a.fs;
  for (int k = a.gptr[g]; k < a.gptr[g + 1]; k++) {
    const int64_t lo = a.cells[k].off, o = so + lo;
    const float A = a.amount[k];
    float sq = 0.f;
    sq = sq + a.Y[0][o];
    sq = sq + a.Y[1][o];
    sq = sq + a.Y[2][o];
    const float beta = a.dtl[lo], alpha = a.dtM[lo] - a.dtl[lo];
    const float sa = sq / (alpha + 3.0f * beta);
    const float corr = A / (alpha + 3.0f * beta), own = A / a.dtM[lo];
    const float im = a.invmu[lo];
    a.gL[o] = a.gL[o] + sa * (3.0f * corr - own) * (beta * beta * a.dtI);
    a.gM[o] = a.gM[o] + sa * (corr - own) * (2.0f * a.dt / (im * im));
  }
}

// k_grad_a2 with wavefield 1 given explicitly (k_adjoint2d.cu)
int grad_a2_launch(Plan *p, const float *p1A, const float *p1B, const float *vx1A, const float *vx1B,
                   const float *vz1A, const float *vz1B);

// ---------------------------------------------------------------------------
// the adjoint run
// ---------------------------------------------------------------------------
static int turn(Plan *p, int s) {
  const int nt = p->d.nt, j = nt - s + 1;
  const int vflags = s < nt ? (1 | 2 | 4) : (1 | 4);
  int rc;
  if (p->d.ndim == 2) {
    const int A = p->cur[0], B = A ^ 1;
    if ((rc = aux_step2(p, s, j))) return rc;
    if ((rc = step_a2_wavefield(p, 0, 0))) return rc;  // A -> B: state s
    if (s < nt && (rc = aux_step2(p, s + 1, j))) return rc;
    if ((rc = step_a2_wavefield(p, 0, vflags))) return rc;  // B -> A: V_{s+1}, A keeps P_{s-1}
    float *const *SA = p->state[A][0], *const *SB = p->state[B][0];
    if ((rc = grad_a2_launch(p, SA[GPI_P], SB[GPI_P], SA[GPI_VX], SB[GPI_VX], SA[GPI_VZ], SB[GPI_VZ]))) return rc;
    return step_a2_wavefield(p, 1, 0);  // adjoint step j
  }
  float *const *W = p->state[0][0], *const *X = p->state[1][0];  // X: scratch copies
  const size_t bytes = p->fstride * p->d.nshots * sizeof(float);
  const int vf[3] = {GPI_VX, GPI_VY, GPI_VZ};
  const bool ela = p->d.physics == GPI_ELASTIC;
  if ((rc = aux_step2(p, s, j))) return rc;
  for (int f = 0; f < NFIELD; f++)  // the stresses (or p) of state s-1
    if (p->present[f] && f != GPI_VX && f != GPI_VY && f != GPI_VZ)
      GPI_CUDA(p, cudaMemcpyAsync(X[f], W[f], bytes, cudaMemcpyDeviceToDevice, p->stream));
  if ((rc = step3_wavefield(p, 0, 0))) return rc;
  if (ela && p->n_cells > 0) {
    GradE3SrcArgs sa;
    sa.fs = p->fstride;
    sa.nshots = p->d.nshots;
    sa.cells = p->d_cells;
    sa.gptr = p->d_group_ptr;
    sa.amount = p->d_amount;
    sa.Y[0] = p->state[0][1][GPI_TAUXX];
    sa.Y[1] = p->state[0][1][GPI_TAUYY];
    sa.Y[2] = p->state[0][1][GPI_TAUZZ];
    sa.dtM = p->coef[6];
    sa.dtl = p->coef[7];
    sa.invmu = p->mod[1];
    sa.gL = p->grad[0];
    sa.gM = p->grad[1];
    sa.dt = (float)p->d.dt;
    sa.dtI = (float)(1.0 / p->d.dt);
    k_grad_e3_src<<<(p->d.nshots + 63) / 64, 64, 0, p->stream>>>(sa);
    p->launches++;
    GPI_CUDA(p, cudaGetLastError());
  }
  for (int d = 0; d < 3; d++)
    GPI_CUDA(p, cudaMemcpyAsync(X[vf[d]], W[vf[d]], bytes, cudaMemcpyDeviceToDevice, p->stream));  // V_s
  if (s < nt && (rc = aux_step2(p, s + 1, j))) return rc;
  if ((rc = step3_wavefield(p, 0, vflags & 3))) return rc;  // V_{s+1} in place
  if (ela) {
    GradE3Args e;
    e.nz = p->d.nz;
    e.ny = p->d.ny;
    e.nx = p->d.nx;
    e.NZP = p->NZP;
    e.NYP = p->NYP;
    e.fs = p->fstride;
    e.nshots = p->d.nshots;
    for (int f = 0; f < NFIELD; f++) {
      e.Y[f] = p->state[0][1][f];
      e.X[f] = X[f];
      e.W[f] = W[f];
    }
    e.dtM = p->coef[6];
    e.dtl = p->coef[7];
    e.invmu = p->mod[1];
    e.gL = p->grad[0];
    e.gM = p->grad[1];
    e.gR = p->grad[2];
    e.dt = (float)p->d.dt;
    e.dtI = (float)(1.0 / p->d.dt);
    k_grad_e3<<<152 * 16, 256, 0, p->stream>>>(e);
    p->launches++;
    GPI_CUDA(p, cudaGetLastError());
    return step3_wavefield(p, 1, 0);  // adjoint step j
  }
  Grad3Args g;
  g.nz = p->d.nz;
  g.ny = p->d.ny;
  g.nx = p->d.nx;
  g.NZP = p->NZP;
  g.NYP = p->NYP;
  g.fs = p->fstride;
  g.nshots = p->d.nshots;
  float *const *Y = p->state[0][1];
  g.p2 = Y[GPI_P];
  g.pold = X[GPI_P];
  g.pnew = W[GPI_P];
  for (int d = 0; d < 3; d++) {
    g.v2[d] = Y[vf[d]];
    g.vs[d] = X[vf[d]];
    g.vs1[d] = W[vf[d]];
  }
  g.gK = p->grad[0];
  g.gR = p->grad[1];
  g.dtI = (float)(1.0 / p->d.dt);
  g.imaging = p->d.imaging;
  k_grad_a3<<<152 * 16, 256, 0, p->stream>>>(g);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return step3_wavefield(p, 1, 0);  // adjoint step j
}

static int advance(Plan *p, int from, int to) {
  for (int s = from + 1; s <= to; s++) {
    int rc = aux_step2(p, s, 0);
    if (!rc) rc = p->d.ndim == 2 ? step_a2_wavefield(p, 0, 0) : step3_wavefield(p, 0, 0);
    if (rc) return rc;
  }
  return GPI_OK;
}

int ckpt_adjoint(Plan *p) {
  if (!p->ck_pool || p->ck_slots <= 0) return fail(p, GPI_E_STATE, "plan has no checkpoint slots");
  if (!p->grad[0] || !p->grad[1]) return fail(p, GPI_E_STATE, "adjoint run without gradient buffers");
  const Sched S = schedule(p->d.nt, p->ck_slots);
  int rc = zero_wavefield(p, 1);
  for (int i = 0; i < p->nmod && !rc; i++)
    rc = cudaMemsetAsync(p->grad[i], 0, p->fstride * p->d.nshots * sizeof(float), p->stream) ? GPI_E_CUDA : 0;
  int held = -2;  // the state the working buffer of wavefield 1 holds (-2: none)
  for (size_t i = 0; i < S.ops.size() && !rc; i++) {
    const Op &o = S.ops[i];
    switch (o.kind) {
      case OP_RESTORE:
        if (held == o.a) break;
        rc = o.slot < 0 ? zero_wavefield(p, 0) : slot_copy(p, o.slot, false);
        held = o.a;
        break;
      case OP_ADVANCE:
        rc = advance(p, o.a, o.b);
        held = o.b;
        break;
      case OP_STORE:
        rc = slot_copy(p, o.slot, true);
        break;
      case OP_TURN:
        rc = turn(p, o.a);
        held = -2;
        break;
    }
  }
  return rc;
}

// the slots each forward_save run fills (called before it)
void ckpt_prepare_forward(Plan *p) { p->ck_first = schedule(p->d.nt, p->ck_slots).first; }

}  // namespace gpi

extern "C" int gpi_checkpoint_schedule(int nt, int slots, int64_t *advances, int64_t *turns, int *stored) {
  if (nt < 1 || slots < 1) return GPI_E_INVALID;
  const gpi::Sched S = gpi::schedule(nt, slots);
  if (advances) *advances = S.advances;
  if (turns) *turns = S.turns;
  if (stored) *stored = (int)S.first.size();
  return GPI_OK;
}
