// k_acoustic2d.cu -- fused 2-D acoustic time step (order 4).
//
// One launch advances every shot by one time step:
//   update_dstress! + update_v! + add_velocity_source!  (velocities to t-1/2)
//   update_dv! + update_stress! + add_stress_source!    (pressure to t)
// which the reference runs as ~12 separate kernels on materialised
// derivative arrays (src/fdtd/advance_acou.jl:11-96, :258-313,
// src/fdtd/cpml.jl:158-215, src/fdtd/dirichlet.jl:1-79,
// src/fdtd/source.jl:61-177).  Index arithmetic follows the reference's
// staggered shapes (src/fields.jl:92-216, src/fdtd/diff2D.jl:47-97):
//   vx[r, c] += cx * D_x(p[r, c-3..c]),  r in 4..nz-3, c in 4..nx
//   vz[q, c] += cz * D_z(p[q-3..q, c]),  q in 4..nz,   c in 4..nx-3
//   p[r, c]  += (D_x(vx[r, c..c+3]) + D_z(vz[r..r+3, c])) * dtK
// with D(a0..a3) = 27 a2 - 27 a1 + a0 - a3 scaled by 1/(24 d).
//
// Work decomposition (same scheme as the elastic kernel): a block owns TZ
// rows x L columns of p of one shot and sweeps its columns; one producer
// thread streams each input column (p over rows z0-4..z0+TZ+3; vx, vz, cx, cz
// over z0..z0+TZ+3; dtK over z0..z0+TZ-1) into an 8-slot shared-memory ring
// with bulk asynchronous copies completing on mbarriers, four columns ahead.
// Interior tiles run a straight-line path; tiles that touch a CPML strip, a
// rigid face or a source run the general path with the CPML memory loaded
// ahead of use.  Halo velocities are recomputed from the input buffer
// (ping-pong state): one HBM pass per step, 36 B per cell update.
#include <algorithm>

#include "k_stencil.cuh"

namespace gpi {

// the fields of one wavefield a launch advances
struct A2W {
  const float *pA, *vxA, *vzA;
  float *pB, *vxB, *vzB;
  const float *psA[4];
  float *psB[4];
  const int32_t *gptr;  // this wavefield's injection-cell groups
};

// the imaging condition of the fused adjoint step (two wavefields: 0 the
// time-reversed modelled field, 1 the adjoint field), compute_gradient!
// (src/fdtd/gradient.jl:17-64):
//   gK += p2_prev (p1_prev - p1) dtI                          (p cells)
//   hx += vx2_prev (vx1 - vx1_prev) dtI, hz likewise           (velocity cells)
// The rho term is linear in the per-step velocity products, so its
// neighbour averages are formed once from hx and hz after the last step
// (k_img_rho) instead of every step.
struct A2Img {
  float *gK, *hx, *hz;
  const float *prev;  // strip values of p1 before boundary_force! (x strips, then z strips)
  int64_t pstride;    // floats per shot in prev
  int nb, npx, npz;   // strip width and PML offsets of the strips
  float dtI;
};

struct A2Args {
  int nz, nx, NZP;
  int64_t fs;
  int npml, faces, rigid;
  float dxI, dzI;
  int nzb;
  A2W w[2];
  int64_t pss[4];
  const float *cx, *cz, *dtK;
  const float *pml;  // [4][3][2*npml]
  const InjCell *cells;
  const float *amount;
  int vonly;  // bit 0: velocity half step only; bit 1: with the velocity
              // sources; bit 2: leave the target p unwritten
  int *err;
  const int4 *tiles;  // (z-block, first column, end column, shot) per block
  int zsw, pzw, psf;  // z-strip column stride, staged window, CPML floats per ring slot and wavefield
  int inj_cap;        // injection cells a block copies to shared memory (0: read from global memory)
  A2Img g;
};

constexpr int A2_TZ = TZ2;        // pressure rows per block
constexpr int A2_THREADS = 128;   // TZ + 3 velocity rows, one per thread
constexpr int A2_R8 = A2_TZ + 8;  // p rows z0-4 .. z0+TZ+3
constexpr int A2_R4 = A2_TZ + 4;  // velocity-input rows z0 .. z0+TZ+3

// Ring slot layout (floats) for NW wavefields: wavefield 0's p | vx | vz,
// the coefficients cx | cz | dtK, then (NW = 2) wavefield 1's p | vx | vz;
// the CPML windows of each wavefield follow.  Every part starts 16-byte
// aligned.  (The imaging accumulators are read by their own threads, one
// column ahead, not staged.)
template <int NW>
struct A2L {
  // 4 columns in use by the stencils plus 4 in flight (deep prefetch for the
  // latency-bound small grids); the fused adjoint keeps 2 in flight (5
  // blocks of interior tiles on an SM) and 1 in its band tiles (5 blocks)
  __host__ __device__ static constexpr int ring(int mode) { return NW == 1 ? 8 : mode == 1 ? 5 : 6; }
  static constexpr int TZ = A2_TZ, R8 = A2_R8, R4 = A2_R4;
  static constexpr int P0 = 0, VX0 = R8, VZ0 = R8 + R4, CX = R8 + 2 * R4, CZ = R8 + 3 * R4, DTK = R8 + 4 * R4;
  static constexpr int SLOT1 = DTK + TZ;
  static constexpr int P1 = SLOT1, VX1 = P1 + R8, VZ1 = VX1 + R4;
  static constexpr int SLOT = NW == 1 ? SLOT1 : VZ1 + R4;
  __host__ __device__ static constexpr int OP(int w) { return w ? P1 : P0; }
  __host__ __device__ static constexpr int OVX(int w) { return w ? VX1 : VX0; }
  __host__ __device__ static constexpr int OVZ(int w) { return w ? VZ1 : VZ0; }
  // shared memory of a block of tile class `mode` with `psf` CPML floats per
  // slot and wavefield and room for `cap` injection cells (column, row,
  // amount)
  static size_t smem(int mode, int psf, int cap) {
    const int RING = ring(mode);
    return 128 + sizeof(float) * (RING * (SLOT + NW * psf) + 2 * NW * RING * R4 + 3 * cap);
  }
};

// CPML floats per ring slot and wavefield of the general kernel: two z-strip
// windows (dpdz, dvzdz) and the x-strip columns of dpdx and dvxdx
inline int a2_psi_floats(const Plan &p) {
  const bool zf = p.d.pml_faces & (GPI_ZMIN | GPI_ZMAX), xf = p.d.pml_faces & (GPI_XMIN | GPI_XMAX);
  return (zf ? 2 * p.pzw : 0) + (xf ? 2 * A2_TZ : 0);
}

// position of p cell (r, c) in the strip block of boundary_save! (x strips
// nz x 2nb, then z strips 2nb x nx), -1 when the cell is in no strip
__device__ __forceinline__ int64_t a2_strip_index(const A2Img &g, int nz, int nx, int r, int c) {
  const int nb = g.nb;
  int j = -1;
  if (c > g.npx && c <= g.npx + nb)
    j = c - g.npx - 1;
  else if (c > nx - g.npx - nb && c <= nx - g.npx)
    j = nb + c - (nx - g.npx - nb) - 1;
  if (j >= 0) return (int64_t)(r - 1) + (int64_t)nz * j;
  if (r > g.npz && r <= g.npz + nb)
    j = r - g.npz - 1;
  else if (r > nz - g.npz - nb && r <= nz - g.npz)
    j = nb + r - (nz - g.npz - nb) - 1;
  if (j >= 0) return (int64_t)nz * 2 * nb + j + (int64_t)2 * nb * (c - 1);
  return -1;
}

// MODE 0: interior tiles (no CPML, face or source: straight-line code);
// MODE 1: tiles away from the x edges and x strips (the band code over every
// column: z strips, z mirrors, sources); MODE 2: the same with x-strip
// columns; MODE 3: tiles with x-edge columns (the band code plus the general
// code for the edge and source columns).
// NW = 1: one wavefield (a.w[0]); NW = 2: the adjoint step of both
// wavefields with the imaging condition (a.g), one pass over the state.
// The body takes the arguments by reference: the kernel's own parameters
// (one plan) or a plan's arguments copied to shared memory (k_a2_batch).
template <int MODE, int NW>
__device__ __forceinline__ void a2_body(const A2Args &a, const int4 tile) {
  using L = A2L<NW>;
  constexpr bool FAST = MODE == 0, XPSI = MODE >= 2, IMG = NW == 2;
  constexpr int TZ = L::TZ, R8 = L::R8, R4 = L::R4, SLOT = L::SLOT, RING = L::ring(MODE);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  float *ring = reinterpret_cast<float *>(smem + 128);  // [RING][SL], layout A2L
  const int PSW = FAST ? 0 : a.psf;                     // CPML floats per slot and wavefield
  const int SL = SLOT + NW * PSW;                       // floats per ring slot
  float *svx = ring + RING * SL;                        // [NW][RING][R4] new velocities
  float *svz = svx + NW * RING * R4;
  __shared__ int s_beg[3 * NW], s_cnt[3 * NW];
  __shared__ int s_err;
  const int t = threadIdx.x;
  const int zb = tile.x, shot = tile.w & 0xffff;  // (the high half: a batch's plan slot)
  const int z0 = 1 + zb * TZ, x0 = tile.y, x1 = tile.z;
  const int xbase = x0 - 3, xlast = x1 + 2;
  const bool lastx = x1 == a.nx + 1, lastz = zb == a.nzb - 1;
  const int nz = a.nz, nx = a.nx, npml = a.npml, NZP = a.NZP;
  const int64_t so = (int64_t)shot * a.fs;
  const bool xlo = a.faces & GPI_XMIN, xhi = a.faces & GPI_XMAX, zlo = a.faces & GPI_ZMIN, zhi = a.faces & GPI_ZMAX;
  const bool rxlo = a.rigid & GPI_XMIN, rxhi = a.rigid & GPI_XMAX, rzlo = a.rigid & GPI_ZMIN, rzhi = a.rigid & GPI_ZMAX;
  const int P6 = 6 * npml;
  auto S = [&](int rr, int cc) -> int64_t { return (int64_t)(cc + XOFF - 1) * NZP + (rr + ZOFF - 1); };
  auto XS = [&](int j, int rr) -> int64_t { return (int64_t)j * NZP + (rr + ZOFF - 1); };
  auto ZS = [&](int cc, int j) -> int64_t { return (int64_t)(cc + XOFF - 1) * a.zsw + j; };
  auto psA = [&](int w, int i) -> const float * { return a.w[w].psA[i] + shot * a.pss[i]; };
  auto psB = [&](int w, int i) -> float * { return a.w[w].psB[i] + shot * a.pss[i]; };
  auto slot = [&](int cc) -> int { return (cc - xbase) % RING; };
  auto SVX = [&](int w, int s) -> float * { return svx + (w * RING + s) * R4; };
  auto SVZ = [&](int w, int s) -> float * { return svz + (w * RING + s) * R4; };
  // General kernel: the CPML memory of each column travels in its ring slot
  // (z-strip windows of dpdz and dvzdz, x-strip columns of dpdx and dvxdx).
  const int zt = FAST ? 0 : zstrip_touch(z0, TZ, nz, npml, zlo, zhi);
  const int zoff = FAST ? 0 : zstrip_off(zt, a.zsw, a.pzw);
  const int PZW = FAST ? 0 : a.pzw;
  // z strip indexed by strip slot (i: 0 dpdz, 1 dvzdz), x strip by row
  // (i: 0 dpdx, 1 dvxdx), by column and by ring slot
  auto PZs = [&](int w, int i, int s) -> const float * { return ring + s * SL + SLOT + w * PSW + i * PZW - zoff; };
  auto PXs = [&](int w, int i, int s) -> const float * {
    return ring + s * SL + SLOT + w * PSW + 2 * PZW + i * TZ - z0;
  };
  auto PZ = [&](int w, int i, int cc) -> const float * { return PZs(w, i, slot(cc)); };
  auto PX = [&](int w, int i, int cc) -> const float * { return PXs(w, i, slot(cc)); };

  if (t == 0) {
    for (int s = 0; s < RING; s++) mbar_init(&bar[s], 4);  // one arrival per warp
    mbar_fence_init();
    s_err = 0;
  }
  // injection cells of the tile's columns [x0, xlast] per cursor (wavefield
  // w; k3: 0 vx, 1 vz, 2 p)
  if (t < 3 * NW) {
    const int w = t / 3, k3 = t - 3 * w;
    const int kind = k3 == 0 ? 0 : k3 == 1 ? 2 : 3;
    const int g = shot * NKIND + kind;
    const int32_t *gp = a.w[w].gptr;
    const int b = first_col(a.cells, gp[g], gp[g + 1], x0);
    s_beg[t] = b;
    s_cnt[t] = first_col(a.cells, b, gp[g + 1], xlast + 1) - b;
  }
  __syncthreads();
  // The cursors walk one column per iteration; the cells of the tile (and
  // this step's amounts) are copied to shared memory once, so that no
  // column waits on a global load of its cells.
  int ioff[3 * NW], itot = 0;
#pragma unroll
  for (int j = 0; j < 3 * NW; j++) ioff[j] = itot, itot += s_cnt[j];
  const bool staged = itot <= a.inj_cap;
  int *s_icol = reinterpret_cast<int *>(svz + NW * RING * R4), *s_irow = s_icol + a.inj_cap;
  float *s_iamt = reinterpret_cast<float *>(s_irow + a.inj_cap);
  if (staged && itot > 0) {
    for (int i = t; i < itot; i += A2_THREADS) {
      int j = 0;
      while (j < 3 * NW - 1 && i >= ioff[j + 1]) j++;
      const int k = s_beg[j] + i - ioff[j];
      s_icol[i] = a.cells[k].col;
      s_irow[i] = a.cells[k].row;
      s_iamt[i] = a.amount[k];
    }
    __syncthreads();
  }
  const InjView iv = staged ? InjView{s_icol, s_irow, s_iamt, 1}
                            : InjView{&a.cells[0].col, &a.cells[0].row, a.amount, (int)(sizeof(InjCell) / sizeof(int))};

  // producers: lane 0 of each warp issues its share of a column's bulk
  // copies and arrives on the slot's mbarrier with the bytes of its share
  // (warp 0 p, warp 1 vx vz, warp 2 cx and the dpdz CPML window, warp 3 cz
  // dtK and the dvzdz window; the x-strip CPML columns on warps 0 and 3;
  // the fused adjoint adds the second wavefield's p on warp 0, its vx on
  // warp 2 and vz on warp 3)
  const int wq = t >> 5;
  const bool issuer = (t & 31) == 0;
  int next = xbase;
  auto issue = [&](int upto) {
    for (; next <= upto && next <= xlast; next++) {
      const int s = slot(next);
      float *sl = ring + s * SL;
      const int64_t oV = S(z0, next);
      int jx = -1;
      if constexpr (XPSI) {
        if (wq == 0) jx = pml_slot(next - 3, nx - 3, npml, xlo, xhi);
        if (wq == 3) jx = pml_slot(next, nx, npml, xlo, xhi);
      }
      uint32_t bytes = wq == 0 ? R8 * 4 : wq == 1 ? 2 * R4 * 4 : wq == 2 ? R4 * 4 : (R4 + TZ) * 4;
      if constexpr (IMG) bytes += wq == 0 ? R8 * 4 : wq == 1 ? 0 : R4 * 4;
      if constexpr (!FAST) {
        if (zt && wq >= 2) bytes += NW * PZW * 4;
        if (jx >= 0) bytes += NW * TZ * 4;
      }
      mbar_expect_tx(&bar[s], bytes);
#pragma unroll
      for (int w = 0; w < NW; w++) {
        if (wq == 0) {
          bulk_g2s(sl + L::OP(w), a.w[w].pA + so + oV - 4, R8 * 4, &bar[s]);
        } else if (wq == 1 && w == 0) {
          bulk_g2s(sl + L::OVX(w), a.w[w].vxA + so + oV, R4 * 4, &bar[s]);
          bulk_g2s(sl + L::OVZ(w), a.w[w].vzA + so + oV, R4 * 4, &bar[s]);
        } else if (w == 1 && wq >= 2) {
          bulk_g2s(sl + (wq == 2 ? L::OVX(w) : L::OVZ(w)), (wq == 2 ? a.w[w].vxA : a.w[w].vzA) + so + oV, R4 * 4,
                   &bar[s]);
        }
        if constexpr (!FAST) {
          float *ps = sl + SLOT + w * PSW;
          if (zt && wq >= 2) bulk_g2s(ps + (wq - 2) * PZW, psA(w, wq == 2 ? 1 : 3) + ZS(next, zoff), PZW * 4, &bar[s]);
          if (jx >= 0) bulk_g2s(ps + 2 * PZW + (wq == 0 ? 0 : TZ), psA(w, wq == 0 ? 0 : 2) + XS(jx, z0), TZ * 4, &bar[s]);
        }
      }
      if (wq == 2) {
        bulk_g2s(sl + L::CX, a.cx + oV, R4 * 4, &bar[s]);
      } else if (wq == 3) {
        bulk_g2s(sl + L::CZ, a.cz + oV, R4 * 4, &bar[s]);
        bulk_g2s(sl + L::DTK, a.dtK + oV, TZ * 4, &bar[s]);
      }
    }
  };
  // interior and band tiles of one wavefield: each issuing lane keeps the
  // source pointers of its share of a column (at most three copies: fields
  // advance by NZP per column, z-strip CPML windows by zsw) and advances
  // them per issue
  constexpr bool PROD = MODE <= 1 && NW == 1;
  const float *fs0 = nullptr, *fs1 = nullptr, *fs2 = nullptr;
  int fd0 = 0, fd1 = 0, fd2 = 0, fst2 = NZP;
  uint32_t fn0 = 0, fn1 = 0, fn2 = 0;
  if constexpr (PROD) {
    const int64_t oV = S(z0, xbase);
    if (wq == 0) {
      fs0 = a.w[0].pA + so + S(z0 - 4, xbase), fd0 = 0, fn0 = R8 * 4;
    } else if (wq == 1) {
      fs0 = a.w[0].vxA + so + oV, fs1 = a.w[0].vzA + so + oV;
      fd0 = R8, fd1 = R8 + R4, fn0 = fn1 = R4 * 4;
    } else if (wq == 2) {
      fs0 = a.cx + oV, fd0 = R8 + 2 * R4, fn0 = R4 * 4;
    } else {
      fs0 = a.cz + oV, fs1 = a.dtK + oV;
      fd0 = R8 + 3 * R4, fd1 = R8 + 4 * R4, fn0 = R4 * 4, fn1 = TZ * 4;
    }
    if (!FAST && zt && wq >= 2) {
      // z-strip CPML windows: warp 2 dpdz, warp 3 dvzdz
      const float *pz = psA(0, wq == 2 ? 1 : 3) + ZS(xbase, zoff);
      const int dz = SLOT + (wq - 2) * PZW;
      if (wq == 2)
        fs1 = pz, fd1 = dz, fn1 = PZW * 4;
      else
        fs2 = pz, fd2 = dz, fn2 = PZW * 4, fst2 = a.zsw;
    }
  }
  const int fst1 = (!FAST && zt && wq == 2) ? a.zsw : NZP;
  // the next column of this warp's share into ring slot sl
  auto issue_fast = [&](int sl) {
    float *d = ring + sl * SL;
    mbar_expect_tx(&bar[sl], fn0 + fn1 + fn2);
    bulk_g2s(d + fd0, fs0, fn0, &bar[sl]);
    if (fn1) bulk_g2s(d + fd1, fs1, fn1, &bar[sl]);
    if (fn2) bulk_g2s(d + fd2, fs2, fn2, &bar[sl]);
    fs0 += NZP, fs1 += fst1, fs2 += fst2;
  };
  if constexpr (PROD) {
    if (issuer)
      for (int sl = 0; sl < RING && xbase + sl <= xlast; sl++) issue_fast(sl);
  } else {
    if (issuer) issue(xbase + RING - 1);
  }
  // column c + RING - 1 into the slot the stencils just released
  auto issue_next = [&](int c, int sl) {
    if constexpr (PROD) {
      if (c + RING - 1 <= xlast) issue_fast(sl);
    } else {
      issue(c + RING - 1);
    }
  };
  auto wait_col = [&](int cc) {
    const int j = cc - xbase;
    if (!mbar_wait(&bar[j % RING], (j / RING) & 1)) s_err = 1;
  };

  InjVCursor cvx[NW], cvz[NW], cst[NW];
#pragma unroll
  for (int w = 0; w < NW; w++) {
    const int j = 3 * w;
    const int b0 = staged ? ioff[j] : s_beg[j], b1 = staged ? ioff[j + 1] : s_beg[j + 1],
              b2 = staged ? ioff[j + 2] : s_beg[j + 2];
    cvx[w].init(iv, b0, b0 + s_cnt[j]);
    cvz[w].init(iv, b1, b1 + s_cnt[j + 1]);
    cst[w].init(iv, b2, b2 + s_cnt[j + 2]);
  }

  // velocity row q (t < TZ, and 3 halo rows for vz); pressure row r
  const int kq = t < TZ + 3 ? t : -1;
  const int q = z0 + kq;
  const bool vact = kq >= 0;
  const bool ownr = kq >= 0 && (kq < TZ || lastz);
  const bool vxr = kq >= 0 && kq < TZ && q >= 4 && q <= nz - 3, vzr = q >= 4 && q <= nz;
  const int jq1 = pml_slot(q - 3, nz - 3, npml, zlo, zhi);  // dpdz (z strip)
  // rows below nz+3 are never stored nor read
  const int gsrc = (rzlo && q <= 2) ? 5 - q : (rzhi && q >= nz + 2 && q <= nz + 3) ? 2 * nz + 3 - q : 0;
  const int r = z0 + t;
  const bool srow = t < TZ && r <= nz;
  const int jr3 = pml_slot(r, nz, npml, zlo, zhi);  // dvzdz (z strip)

  for (int cc = xbase; cc < x0 && cc <= xlast; cc++) wait_col(cc);

  // imaging condition (NW = 2): wavefield 0's new values, the old values of
  // both wavefields from ring slot s (row index k); the accumulators of the
  // iteration's own cells (velocity row q of column c + 3, pressure row r of
  // column c) are loaded by their threads one iteration ahead (n*) and used
  // from a*; p1_prev is the unforced value where boundary_force! replaced it
  const float dtI = IMG ? a.g.dtI : 0.f;
  float ahx = 0.f, ahz = 0.f, agk = 0.f, app = 0.f, nhx = 0.f, nhz = 0.f, ngk = 0.f, npp = 0.f;
  bool apv = false, npv = false;
  auto img_load = [&](int c) {
    if constexpr (IMG) {
      const int64_t o3 = so + S(q, c + 3), o0 = so + S(r, c);
      nhx = a.g.hx[o3];
      nhz = a.g.hz[o3];
      ngk = a.g.gK[o0];
      if constexpr (!FAST) {
        const int64_t si = srow ? a2_strip_index(a.g, nz, nx, r, c) : -1;
        npv = si >= 0;
        npp = npv ? a.g.prev[shot * a.g.pstride + si] : 0.f;
      }
    }
  };
  // at the top of iteration c: its accumulators, and the next iteration's loads
  auto img_next = [&](int c) {
    if constexpr (IMG) {
      ahx = nhx, ahz = nhz, agk = ngk, app = npp, apv = npv;
      img_load(c + 1);
    }
  };
  auto img_vx = [&](int s, int k, int64_t o, float vx1, float h) {
    const float *cs = ring + s * SL;
    a.g.hx[o] = h + cs[L::VX1 + k] * (vx1 - cs[L::VX0 + k]) * dtI;
  };
  auto img_vz = [&](int s, int k, int64_t o, float vz1) {
    const float *cs = ring + s * SL;
    a.g.hz[o] = ahz + cs[L::VZ1 + k] * (vz1 - cs[L::VZ0 + k]) * dtI;
  };
  auto img_p = [&](int s, int k, int64_t o, float p1) {
    const float *cs = ring + s * SL;
    const float pp = !FAST && apv ? app : cs[L::P0 + k + 4];
    a.g.gK[o] = agk + cs[L::P1 + k + 4] * (pp - p1) * dtI;
  };
  img_load(xbase);

  // CPML: psi' = b psi + a D ; D' = D kI + psi'  (profile [a | b | kI])
  auto cpml_p = [&](float D, int q4, int j, float psi_old, float *dst, bool own) -> float {
    const float *cf = a.pml + q4 * P6;
    const float psi = __ldg(cf + 2 * npml + j) * psi_old + __ldg(cf + j) * D;
    if (own) *dst = psi;
    return D * __ldg(cf + 4 * npml + j) + psi;
  };
  // the z-strip profile of this thread's rows, loaded once
  auto zprof = [&](int q4, int j) -> float3 {
    if (FAST || j < 0) return make_float3(0.f, 0.f, 0.f);
    const float *cf = a.pml + q4 * P6;
    return make_float3(__ldg(cf + j), __ldg(cf + 2 * npml + j), __ldg(cf + 4 * npml + j));
  };
  const float3 cq1 = zprof(1, jq1), cr3 = zprof(3, jr3);
  auto cpml_z = [&](float D, float3 cf, float psi_old, float *dst, bool own) -> float {
    const float psi = cf.y * psi_old + cf.x * D;
    if (own) *dst = psi;
    return D * cf.z + psi;
  };
  // the same as selects: the memory variable applies where `on`
  auto cpml_zs = [&](float D, float3 cf, float psi_old, bool on, float *dst, bool own) -> float {
    const float psi = cf.y * psi_old + cf.x * D;
    if (on && own) *dst = psi;
    return on ? D * cf.z + psi : D;
  };
  auto cpml_xs = [&](float D, int q4, int j, float psi_old, bool on, float *dst, bool own) -> float {
    const float *cf = a.pml + q4 * P6;
    const float psi = __ldg(cf + 2 * npml + j) * psi_old + __ldg(cf + j) * D;
    if (on && own) *dst = psi;
    return on ? D * __ldg(cf + 4 * npml + j) + psi : D;
  };

  // the interior code: every row inside every update domain, no CPML, no
  // face, no source (interior tiles); global offsets of this thread's rows, advanced one column per
  // iteration: velocities of column xbase+3+it, pressure of column xbase+it
  int64_t ov = so + S(q, xbase + 3), os = so + S(r, xbase);
  // velocities of column cc from ring slots s3..s0 = columns cc-3..cc
  auto vel_fast = [&](int w, int cc, int s3, int s2, int s1, int s0) {
    if (!vact) return;
    const int k = kq, kk = kq + 4;
    const float *cs = ring + s0 * SL, *pc = cs + L::OP(w);
    const float vz = cs[L::OVZ(w) + k] + cs[L::CZ + k] * (st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI);
    SVZ(w, s0)[k] = vz;
    if (kq < TZ) {
      const float *p3 = ring + s3 * SL + L::OP(w), *p2 = ring + s2 * SL + L::OP(w), *p1 = ring + s1 * SL + L::OP(w);
      const float vx = cs[L::OVX(w) + k] + cs[L::CX + k] * (st4(p3[kk], p2[kk], p1[kk], pc[kk]) * a.dxI);
      SVX(w, s0)[k] = vx;
      if (cc < x1) {
        a.w[w].vxB[ov] = vx;
        a.w[w].vzB[ov] = vz;
        if (IMG && w == 0) {
          img_vx(s0, k, ov, vx, ahx);
          img_vz(s0, k, ov, vz);
        }
      }
    }
  };
  // pressure of column c from velocity slots s0..s3 = columns c..c+3 (the
  // velocity half step: the old pressure, or nothing with vonly bit 2)
  auto str_fast = [&](int w, int c, int s0, int s1, int s2, int s3) {
    if (t >= TZ) return;
    const int k = t;
    const float *cs = ring + s0 * SL, *pc = cs + L::OP(w);
    if (a.vonly) {
      if (!(a.vonly & 4)) a.w[w].pB[os] = pc[k + 4];
      return;
    }
    const float *vz = SVZ(w, s0);
    const float Dx = st4(SVX(w, s0)[k], SVX(w, s1)[k], SVX(w, s2)[k], SVX(w, s3)[k]) * a.dxI;
    const float Dz = st4(vz[k], vz[k + 1], vz[k + 2], vz[k + 3]) * a.dzI;
    const float pn = pc[k + 4] + (Dx + Dz) * cs[L::DTK + k];
    a.w[w].pB[os] = pn;
    if (IMG && w == 0) img_p(s0, k, os, pn);
  };

  // Dispatch per warp and per column: a warp runs the straight-line code
  // unless one of its rows or the current column touches a CPML strip, a
  // rigid face, a domain edge or a source cell.
  if constexpr (FAST) {
    // interior tile: inside every update domain, no CPML, no face, no
    // source.
    // iteration it handles column c = xbase + it: slot(c + m) = (it + m) %
    // RING; unrolled by RING so that every slot index is a constant (base is
    // a multiple of RING; a slot's mbarrier parity flips once per RING
    // columns)
    // (the fused step's loop body is twice as long: rolled, so that the
    // code stays within the instruction cache)
    const int ncol = x1 - xbase;
    if constexpr (NW == 1) {
      for (int base = 0; base < ncol; base += RING) {
        const uint32_t ph = (uint32_t)(base / RING) & 1u;
#pragma unroll
        for (int u = 0; u < RING; u++) {
          const int it = base + u;
          if (it >= ncol) break;
          const int c = xbase + it;
          if (!mbar_wait(&bar[(u + 3) % RING], ph ^ (uint32_t)((u + 3) / RING))) s_err = 1;
          vel_fast(0, c + 3, u % RING, (u + 1) % RING, (u + 2) % RING, (u + 3) % RING);
          __syncthreads();
          if (issuer && it >= 1) issue_next(c, (u + RING - 1) % RING);
          if (c >= x0) str_fast(0, c, u % RING, (u + 1) % RING, (u + 2) % RING, (u + 3) % RING);
          ov += NZP, os += NZP;
        }
      }
    } else {
      for (int it = 0; it < ncol; it++) {
        const int c = xbase + it;
        const int s0 = it % RING, s1 = (it + 1) % RING, s2 = (it + 2) % RING, s3 = (it + 3) % RING;
        img_next(c);
        if (!mbar_wait(&bar[s3], ((it + 3) / RING) & 1)) s_err = 1;
#pragma unroll
        for (int w = 0; w < NW; w++) vel_fast(w, c + 3, s0, s1, s2, s3);
        __syncthreads();
        if (issuer) issue(c + RING - 1);
        if (c >= x0) {
#pragma unroll
          for (int w = 0; w < NW; w++) str_fast(w, c, s0, s1, s2, s3);
        }
        ov += NZP, os += NZP;
      }
    }
  } else {
  // columns that need the full general code: x edges and mirrors, sources
  auto colfull_v = [&](int cc) { return a.vonly || cc <= 4 || cc >= nx - 4; };
  const bool vsrc = !(a.vonly & 1) || (a.vonly & 2);
  auto colfull_s = [&](int c) { return a.vonly || c >= nx - 4; };
  // per-row constants of the band path (vxr already excludes the halo rows)
  const int kqc = vact ? kq : 0;
  const bool vzb = vact && vzr;
  const int jq1v = vzb ? jq1 : -1, jr3v = srow ? jr3 : -1;
  // in-window strip slots to read when a row is outside its strip
  const int jq1c = jq1v >= 0 ? jq1v : zoff, jr3c = jr3v >= 0 ? jr3v : zoff;
  // warps with a z-strip row (velocity / pressure rows): the others skip the
  // memory-variable code as a whole
  const bool wzv = __any_sync(0xffffffffu, jq1v >= 0), wzs = __any_sync(0xffffffffu, jr3v >= 0);
  // ghost rows of vz (dirichletzmin!/zmax!) read their mirror source from
  // the lane that computes it, when that lane is in the same warp
  const int lane = t & 31;
  const int gdl = gsrc ? gsrc - q : 0;
  const bool gok = lane + gdl >= 0 && lane + gdl < 32;
  const int glane = gok ? lane + gdl : lane;
  const bool gany = __any_sync(0xffffffffu, gsrc != 0);
  {
    // vz of wavefield w at row qq of column cc before its source (source of
    // a mirror row)
    auto vz_any = [&](int w, int qq, int cc) -> float {
      const int kv = qq - z0;
      const float *cs = ring + slot(cc) * SL, *pc = cs + L::OP(w);
      float v = cs[L::OVZ(w) + kv];
      if (qq >= 4 && qq <= nz && cc >= 4 && cc <= nx - 3) {
        const int kk = kv + 4;
        float D = st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI;
        const int j = pml_slot(qq - 3, nz - 3, npml, zlo, zhi);
        if (j >= 0) D = cpml_p(D, 1, j, PZ(w, 0, cc)[j], nullptr, false);
        v = v + cs[L::CZ + kv] * D;
      }
      return v;
    };
    // Columns away from the x edges and from sources: every row in one
    // pass; rows outside an update domain keep their value, CPML terms where
    // a strip is met (psi staged in the ring slot of the column)
    // velocities of column cc from ring slots s3..s0 = columns cc-3..cc
    // (cells of the column's vx / vz sources in [ib0, ie0) / [ib1, ie1))
    auto vel_band = [&](int w, int cc, int s3, int s2, int s1, int s0, int ib0, int ie0, int ib1, int ie1) {
      const int k = kqc, kk = kqc + 4, s = s0;
      const float *cs = ring + s * SL, *pc = cs + L::OP(w);
      const float *p3 = ring + s3 * SL + L::OP(w), *p2 = ring + s2 * SL + L::OP(w), *p1s = ring + s1 * SL + L::OP(w);
      const bool ownc = cc < x1;
      const bool ownx = ownc && ownr && q <= nz, ownz = ownc && ownr && q <= nz + 3;
      // branch-free: every row computes its derivatives; rows outside an
      // update domain keep their value, rows outside a strip their plain
      // derivative (selects)
      float Dz = st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI;
      float Dx = st4(p3[kk], p2[kk], p1s[kk], pc[kk]) * a.dxI;
      if (wzv) Dz = cpml_zs(Dz, cq1, PZs(w, 0, s)[jq1c], jq1v >= 0, psB(w, 1) + ZS(cc, jq1c), ownc && ownr);
      if constexpr (XPSI) {
        const int j0 = pml_slot(cc - 3, nx - 3, npml, xlo, xhi);
        if (j0 >= 0) Dx = cpml_xs(Dx, 0, j0, PXs(w, 0, s)[q], vxr, psB(w, 0) + XS(j0, q), ownx);
      }
      float vz = vzb ? cs[L::OVZ(w) + k] + cs[L::CZ + k] * Dz : cs[L::OVZ(w) + k];
      float vx = vxr ? cs[L::OVX(w) + k] + cs[L::CX + k] * Dx : cs[L::OVX(w) + k];
      if (gany) {
        const float g = __shfl_sync(0xffffffffu, vz, glane);
        if (gsrc) vz = gok ? -g : -vz_any(w, gsrc, cc);
      }
      // add_velocity_source! (after the mirrors took their values)
      if (ib0 < ie0) inject(iv, ib0, ie0, q, vx);
      if (ib1 < ie1) inject(iv, ib1, ie1, q, vz);
      if (vact) SVZ(w, s)[k] = vz;
      if (vact && kq < TZ) SVX(w, s)[k] = vx;
      const int64_t o = so + S(q, cc);
      if (ownz) {
        a.w[w].vzB[o] = vz;
        if (IMG && w == 0) img_vz(s, k, o, vz);
      }
      if (ownx && kq < TZ) {
        a.w[w].vxB[o] = vx;
        if (IMG && w == 0) img_vx(s, k, o, vx, ahx);
      }
    };
    // pressure of column c from velocity slots s0..s3 = columns c..c+3;
    // halo lanes recompute the last row and store nothing
    // (cells of the column's pressure sources in [bs, es))
    auto str_band = [&](int w, int c, int s0, int s1, int s2, int s3, int bs, int es) {
      const int k = t < TZ ? t : TZ - 1, rk = z0 + k;
      const float *cs = ring + s0 * SL, *pc = cs + L::OP(w);
      float Dx = st4(SVX(w, s0)[k], SVX(w, s1)[k], SVX(w, s2)[k], SVX(w, s3)[k]) * a.dxI;
      const float *vz = SVZ(w, s0);
      float Dz = st4(vz[k], vz[k + 1], vz[k + 2], vz[k + 3]) * a.dzI;
      if constexpr (XPSI) {
        const int j2 = pml_slot(c, nx, npml, xlo, xhi);
        if (j2 >= 0) Dx = cpml_xs(Dx, 2, j2, PXs(w, 1, s0)[rk], srow, psB(w, 2) + XS(j2, rk), true);
      }
      if (wzs) Dz = cpml_zs(Dz, cr3, PZs(w, 1, s0)[jr3c], jr3v >= 0, psB(w, 3) + ZS(c, jr3c), true);
      float pn = pc[k + 4] + (Dx + Dz) * cs[L::DTK + k];
      if (bs < es) inject(iv, bs, es, r, pn);  // add_stress_source!
      if (srow) {
        a.w[w].pB[so + S(r, c)] = pn;
        if (IMG && w == 0) img_p(s0, k, so + S(r, c), pn);
      }
    };
    if constexpr (MODE == 1 || MODE == 2) {
      // iteration it handles column c = xbase + it: slot(c + m) = (it + m) %
      // RING (a rolled loop: the band code unrolled by the ring length
      // overflows the instruction cache)
      const int ncol = x1 - xbase;
      for (int it = 0; it < ncol; it++) {
        const int c = xbase + it, cc = c + 3;
        img_next(c);
        int ib0[NW], ie0[NW], ib1[NW], ie1[NW], bs[NW], es[NW];
#pragma unroll
        for (int w = 0; w < NW; w++) {
          cvx[w].range(iv, cc, ib0[w], ie0[w]);
          cvz[w].range(iv, cc, ib1[w], ie1[w]);
          bs[w] = es[w] = 0;
          if (c >= x0) cst[w].range(iv, c, bs[w], es[w]);
        }
        if (!mbar_wait(&bar[(it + 3) % RING], ((it + 3) / RING) & 1)) s_err = 1;
#pragma unroll
        for (int w = 0; w < NW; w++)
          vel_band(w, cc, it % RING, (it + 1) % RING, (it + 2) % RING, (it + 3) % RING, ib0[w], ie0[w], ib1[w], ie1[w]);
        __syncthreads();
        if (issuer && it >= 1) issue_next(c, (it + RING - 1) % RING);
        if (c >= x0) {
#pragma unroll
          for (int w = 0; w < NW; w++)
            str_band(w, c, it % RING, (it + 1) % RING, (it + 2) % RING, (it + 3) % RING, bs[w], es[w]);
        }
      }
    } else {
      float vpre[NW];  // vx[r, nx] before its source (xmax mirror)
#pragma unroll
      for (int w = 0; w < NW; w++) vpre[w] = 0.f;
      auto vel_edge = [&](int w, int cc, int ib0, int ie0, int ib1, int ie1) {
        if (!vact) return;
        const int k = kq, kk = kq + 4, s = slot(cc);
        const float *cs = ring + s * SL, *pc = cs + L::OP(w);
        const bool ownc = cc >= x0 && (cc < x1 || lastx);
        if (kq < TZ) {
          const bool ownx = ownc && ownr && q <= nz;
          float vx;
          if (rxhi && cc >= nx + 2) {
            vx = cc == nx + 3 ? -vpre[w] : -SVX(w, slot(cc - 1))[k];  // vx[nx+3] = -vx[nx], vx[nx+2] = -vx[nx+1]
          } else {
            vx = cs[L::OVX(w) + k];
            if (vxr && cc >= 4 && cc <= nx) {
              const float *p3 = ring + slot(cc - 3) * SL + L::OP(w), *p2 = ring + slot(cc - 2) * SL + L::OP(w),
                          *p1 = ring + slot(cc - 1) * SL + L::OP(w);
              float D = st4(p3[kk], p2[kk], p1[kk], pc[kk]) * a.dxI;
              const int j0 = pml_slot(cc - 3, nx - 3, npml, xlo, xhi);
              if (j0 >= 0) D = cpml_p(D, 0, j0, PX(w, 0, cc)[q], psB(w, 0) + XS(j0, q), ownx);
              vx = vx + cs[L::CX + k] * D;
            }
            if (cc == nx) vpre[w] = vx;
          }
          if (rxlo && cc == 4) {
            // dirichletxmin!: vx[1] = -vx[4] (before its source), vx[2] = -vx[3]
            const float g1 = -vx, g2 = -SVX(w, slot(3))[k];
            SVX(w, slot(1))[k] = g1;
            SVX(w, slot(2))[k] = g2;
            if (x0 == 1 && ownr && q <= nz) {
              a.w[w].vxB[so + S(q, 1)] = g1;
              a.w[w].vxB[so + S(q, 2)] = g2;
              if (IMG && w == 0) {
                img_vx(slot(1), k, so + S(q, 1), g1, a.g.hx[so + S(q, 1)]);
                img_vx(slot(2), k, so + S(q, 2), g2, a.g.hx[so + S(q, 2)]);
              }
            }
          }
          if (vsrc) inject(iv, ib0, ie0, q, vx);
          SVX(w, s)[k] = vx;
          if (ownx) {
            a.w[w].vxB[so + S(q, cc)] = vx;
            if (IMG && w == 0) img_vx(s, k, so + S(q, cc), vx, ahx);
          }
        }
        float vz;
        if (gsrc) {
          vz = -vz_any(w, gsrc, cc);  // dirichletzmin!/zmax!
        } else {
          vz = cs[L::OVZ(w) + k];
          if (vzr && cc >= 4 && cc <= nx - 3) {
            float D = st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI;
            if (jq1 >= 0) D = cpml_z(D, cq1, PZ(w, 0, cc)[jq1], psB(w, 1) + ZS(cc, jq1), ownc && ownr && cc <= nx);
            vz = vz + cs[L::CZ + k] * D;
          }
        }
        if (vsrc) inject(iv, ib1, ie1, q, vz);
        SVZ(w, s)[k] = vz;
        if (ownc && ownr && cc <= nx && q <= nz + 3) {
          a.w[w].vzB[so + S(q, cc)] = vz;
          if (IMG && w == 0) img_vz(s, k, so + S(q, cc), vz);
        }
      };
      auto str_edge = [&](int w, int c, int bs, int es) {
        if (!srow) return;
        const int k = t, s = slot(c);
        const float *cs = ring + s * SL, *pc = cs + L::OP(w);
        float pn = pc[k + 4];
        if (!a.vonly) {
          float Dx = st4(SVX(w, slot(c))[k], SVX(w, slot(c + 1))[k], SVX(w, slot(c + 2))[k], SVX(w, slot(c + 3))[k]) *
                     a.dxI;
          const int j2 = pml_slot(c, nx, npml, xlo, xhi);
          if (j2 >= 0) Dx = cpml_p(Dx, 2, j2, PX(w, 1, c)[r], psB(w, 2) + XS(j2, r), true);
          const float *vz = SVZ(w, s);
          float Dz = st4(vz[k], vz[k + 1], vz[k + 2], vz[k + 3]) * a.dzI;
          if (jr3 >= 0) Dz = cpml_z(Dz, cr3, PZ(w, 1, c)[jr3], psB(w, 3) + ZS(c, jr3), true);
          pn = pn + (Dx + Dz) * cs[L::DTK + k];
          inject(iv, bs, es, r, pn);  // add_stress_source!
        }
        if (!(a.vonly & 4)) {
          a.w[w].pB[so + S(r, c)] = pn;
          if (IMG && w == 0) img_p(s, k, so + S(r, c), pn);
        }
      };
      // one sweep: iterations c < x0 only compute the first velocity columns
      for (int c = x0 - 3; c < x1; c++) {
        const int cc = c + 3;
        img_next(c);
        int ib0[NW], ie0[NW], ib1[NW], ie1[NW], bs[NW], es[NW];
        bool gv[NW], gs[NW];
#pragma unroll
        for (int w = 0; w < NW; w++) {
          cvx[w].range(iv, cc, ib0[w], ie0[w]);
          cvz[w].range(iv, cc, ib1[w], ie1[w]);
          bs[w] = es[w] = 0;
          if (c >= x0) cst[w].range(iv, c, bs[w], es[w]);
          // general code for x edges, mirrors and sources (block-uniform);
          // otherwise the band code over every row
          gv[w] = colfull_v(cc) || ib0[w] < ie0[w] || ib1[w] < ie1[w];
          gs[w] = colfull_s(c) || bs[w] < es[w];
        }
        wait_col(cc);
#pragma unroll
        for (int w = 0; w < NW; w++) {
          if (gv[w])
            vel_edge(w, cc, ib0[w], ie0[w], ib1[w], ie1[w]);
          else
            vel_band(w, cc, slot(cc - 3), slot(cc - 2), slot(cc - 1), slot(cc), ib0[w], ie0[w], ib1[w], ie1[w]);
        }
        __syncthreads();
        if (issuer) issue(c + RING - 1);
        if (c >= x0) {
#pragma unroll
          for (int w = 0; w < NW; w++) {
            if (gs[w])
              str_edge(w, c, bs[w], es[w]);
            else
              str_band(w, c, slot(c), slot(c + 1), slot(c + 2), slot(c + 3), bs[w], es[w]);
          }
        }
      }
    }
  }
  }
  __syncthreads();
  if (s_err && t == 0) {
    for (int cc = max(xbase, xlast - (RING - 1)); cc <= xlast; cc++) {
      const int j = cc - xbase;
      mbar_wait(&bar[j % RING], (j / RING) & 1);
    }
    atomicExch(a.err, 1);
  }
}

template <int MODE, int NW>
__global__ void __launch_bounds__(A2_THREADS, NW == 2 ? (MODE <= 1 ? 5 : 3) : (MODE == 0 ? 6 : MODE == 1 ? 5 : 4))
    k_a2(const A2Args a) {
  a2_body<MODE, NW>(a, a.tiles[blockIdx.x]);
}

// One step of several plans in one launch (a batch, gpi_batch.cu): the
// tiles of every plan of one class, each tagged with its plan's slot in the
// high half of .w; the block copies its plan's arguments for this class and
// buffer parity (args[(slot * 4 + MODE) * 2 + par]) to shared memory.
template <int MODE>
__global__ void __launch_bounds__(A2_THREADS, MODE == 0 ? 6 : MODE == 1 ? 5 : 4)
    k_a2_batch(const A2Args *__restrict__ args, const int4 *__restrict__ tiles, int par) {
  __shared__ __align__(16) A2Args sa;
  const int4 tile = tiles[blockIdx.x];
  const int slot = tile.w >> 16;
  const int *src = reinterpret_cast<const int *>(args + ((int64_t)slot * 4 + MODE) * 2 + par);
  int *dst = reinterpret_cast<int *>(&sa);
  for (int i = threadIdx.x; i < (int)(sizeof(A2Args) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  a2_body<MODE, 1>(sa, tile);
}

int step_acoustic2d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  if (mode == GPI_ADJOINT && !vonly) return step_adjoint_acoustic2d(p, it);
  (void)ipw_mask;
  (void)it;
  return step_a2_wavefield(p, 0, vonly);
}

// the arguments of one time step of wavefield ipw (nw = 1: 0 the modelled,
// 1 the adjoint wavefield; `flip` swaps its buffers) or of both wavefields
// with the imaging condition (nw = 2)
static void a2_fill(Plan *p, int nw, int ipw, int vonly, int flip, A2Args &a) {
  a.nz = p->d.nz;
  a.nx = p->d.nx;
  a.NZP = p->NZP;
  a.fs = p->fstride;
  a.npml = p->d.npml;
  a.faces = p->d.pml_faces;
  a.rigid = p->d.rigid_faces;
  a.dxI = (float)(1.0 / (p->d.dx * 24.0));
  a.dzI = (float)(1.0 / (p->d.dz * 24.0));
  a.nzb = p->nzb;
  a.w[1] = A2W{};
  for (int w = 0; w < nw; w++) {
    const int pw = nw == 2 ? w : ipw;
    const int A = p->cur[pw] ^ flip, B = A ^ 1;
    A2W &f = a.w[w];
    f.pA = p->state[A][pw][GPI_P];
    f.vxA = p->state[A][pw][GPI_VX];
    f.vzA = p->state[A][pw][GPI_VZ];
    f.pB = p->state[B][pw][GPI_P];
    f.vxB = p->state[B][pw][GPI_VX];
    f.vzB = p->state[B][pw][GPI_VZ];
    for (int q = 0; q < 4; q++) {
      f.psA[q] = p->psi[A][pw][q];
      f.psB[q] = p->psi[B][pw][q];
    }
    f.gptr = p->d_group_ptr + (int64_t)pw * p->d.nshots * NKIND;  // this wavefield's cell groups
  }
  for (int q = 0; q < 4; q++) a.pss[q] = p->psi_stride[q];
  a.cx = p->coef[0];
  a.cz = p->coef[1];
  a.dtK = p->coef[2];
  a.pml = p->pml;
  a.cells = p->d_cells;
  a.amount = p->d_amount;
  a.vonly = vonly;
  a.err = p->d_err;
  a.tiles = p->d_tiles;
  a.zsw = p->zsw;
  a.pzw = p->pzw;
  a.psf = 0;
  a.inj_cap = 0;
  a.g = A2Img{};
  if (nw == 2) {
    a.g.gK = p->grad[0];
    a.g.hx = p->img[0];
    a.g.hz = p->img[1];
    a.g.prev = p->bprev;
    a.g.pstride = p->bstep;
    a.g.nb = p->d.nbound;
    a.g.npx = (p->d.pml_faces & GPI_XMIN) ? p->d.npml : 0;
    a.g.npz = (p->d.pml_faces & GPI_ZMIN) ? p->d.npml : 0;
    a.g.dtI = (float)(1.0 / p->d.dt);
  }
}

// per tile class: CPML floats per ring slot and wavefield, room for the
// injection cells of the largest tile (tiles with more than 2048 read them
// from global memory), shared memory per block
static void a2_sizes(const Plan *p, int nw, int ipw, int vonly, int psf[4], int cap[4], size_t smem[4]) {
  const bool zf = p->d.pml_faces & (GPI_ZMIN | GPI_ZMAX);
  psf[0] = 0;
  psf[1] = zf ? 2 * p->pzw : 0;
  psf[2] = psf[3] = a2_psi_floats(*p);
  for (int m = 0; m < 4; m++) cap[m] = p->inj_tile[nw == 2 ? 2 : ipw][m];
  if (vonly) cap[3] = std::max(cap[3], std::max(cap[1], cap[2]));  // every non-interior tile runs class 3's code
  for (int m = 0; m < 4; m++) {
    if (cap[m] > 2048) cap[m] = 0;
    smem[m] = nw == 1 ? A2L<1>::smem(m, psf[m], cap[m]) : A2L<2>::smem(m, psf[m], cap[m]);
  }
}

// one time step of wavefield ipw (nw = 1) or of both wavefields with the
// imaging condition (nw = 2)
static int a2_launch(Plan *p, int nw, int ipw, int vonly) {
  A2Args a;
  a2_fill(p, nw, ipw, vonly, 0, a);
  int psf[4], cap[4];
  size_t smem[4];
  a2_sizes(p, nw, ipw, vonly, psf, cap, smem);
  void (*const fn1[4])(A2Args) = {k_a2<0, 1>, k_a2<1, 1>, k_a2<2, 1>, k_a2<3, 1>};
  void (*const fn2[4])(A2Args) = {k_a2<0, 2>, k_a2<1, 2>, k_a2<2, 2>, k_a2<3, 2>};
  void (*const *fn)(A2Args) = nw == 1 ? fn1 : fn2;
  for (int m = 0; m < 4; m++)
    if (int rc = ensure_smem_attr(p, (const void *)fn[m], (nw == 1 ? 0 : 8) + m, smem[m])) return rc;
  auto launch = [&](int m, int first, int n, cudaStream_t st) {
    if (n <= 0) return;
    A2Args g = a;
    g.tiles = p->d_tiles + first;
    g.psf = psf[m];
    g.inj_cap = cap[m];
    fn[m]<<<n, A2_THREADS, smem[m], st>>>(g);
    p->launches++;
  };
  const int *n = p->n_tiles;
  const int ntot = n[0] + n[1] + n[2] + n[3];
  if (vonly) {
    // the velocity half step: interior tiles on the interior code (they
    // hold no source), every other tile on the general code
    const int nside = n[0] > 0 && ntot > n[0] ? 1 : 0;
    cudaStream_t st[Plan::NSIDE] = {p->stream, p->stream, p->stream};
    if (int rc = fork_side(p, nside, st)) return rc;
    launch(3, n[0], ntot - n[0], st[0]);
    launch(0, 0, n[0], p->stream);
    GPI_CUDA(p, cudaGetLastError());
    if (int rc = join_side(p, nside)) return rc;
  } else {
    // edge, x-band and band blocks (longer) go first, on their own streams,
    // so that interior blocks fill the SMs around them and their tails
    const int groups = (n[0] > 0) + (n[1] > 0) + (n[2] > 0) + (n[3] > 0);
    const int nside = groups > 1 ? Plan::NSIDE : 0;
    cudaStream_t st[Plan::NSIDE] = {p->stream, p->stream, p->stream};
    if (int rc = fork_side(p, nside, st)) return rc;
    launch(3, n[0] + n[1] + n[2], n[3], st[0]);
    launch(2, n[0] + n[1], n[2], st[1]);
    launch(1, n[0], n[1], st[2]);
    launch(0, 0, n[0], p->stream);
    GPI_CUDA(p, cudaGetLastError());
    if (int rc = join_side(p, nside)) return rc;
  }
  GPI_CUDA(p, cudaGetLastError());
  for (int w = 0; w < nw; w++) p->cur[nw == 2 ? w : ipw] ^= 1;
  return GPI_OK;
}

int step_a2_wavefield(Plan *p, int ipw, int vonly) { return a2_launch(p, 1, ipw, vonly); }

// --- batches of one-wavefield plans (gpi_batch.cu) ---
size_t a2_args_bytes() { return sizeof(A2Args); }

// a forward plan's arguments per tile class and buffer parity ([class][parity],
// parity 1 with the buffers swapped) and its shared memory per class
void a2_batch_args(Plan *p, void *out, size_t smem[4]) {
  int psf[4], cap[4];
  a2_sizes(p, 1, 0, 0, psf, cap, smem);
  A2Args *o = static_cast<A2Args *>(out);
  for (int m = 0; m < 4; m++)
    for (int par = 0; par < 2; par++) {
      A2Args &a = o[m * 2 + par];
      a2_fill(p, 1, 0, 0, par, a);
      a.tiles = nullptr;
      a.psf = psf[m];
      a.inj_cap = cap[m];
    }
}

// one launch of tile class m over n tagged tiles of the batch's plans
int a2_batch_launch(Plan *p, int m, const void *args, const int4 *tiles, int n, int par, size_t smem, cudaStream_t st) {
  void (*const fn[4])(const A2Args *, const int4 *, int) = {k_a2_batch<0>, k_a2_batch<1>, k_a2_batch<2>,
                                                             k_a2_batch<3>};
  if (int rc = ensure_smem_attr(p, (const void *)fn[m], 16 + m, smem)) return rc;
  if (n <= 0) return GPI_OK;  // (n = 0: only the kernel's shared-memory attribute)
  fn[m]<<<n, A2_THREADS, smem, st>>>(static_cast<const A2Args *>(args), tiles, par);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// the adjoint step of both wavefields with the imaging condition in one pass
int step_a2_adjoint_fused(Plan *p) { return a2_launch(p, 2, 0, 0); }

}  // namespace gpi
