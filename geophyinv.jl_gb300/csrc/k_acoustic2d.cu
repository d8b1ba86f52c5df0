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
#include "k_stencil.cuh"

namespace gpi {

struct A2Args {
  int nz, nx, NZP;
  int64_t fs;
  int npml, faces, rigid;
  float dxI, dzI;
  int nzb;
  const float *pA, *vxA, *vzA;
  float *pB, *vxB, *vzB;
  const float *psA[4];
  float *psB[4];
  int64_t pss[4];
  const float *cx, *cz, *dtK;
  const float *pml;  // [4][3][2*npml]
  const InjCell *cells;
  const int32_t *gptr;
  const float *amount;
  int vonly;  // bit 0: velocity half step only; bit 1: with the velocity
              // sources; bit 2: leave the target p unwritten
  int *err;
  const int4 *tiles;  // (z-block, first column, end column, shot) per block
  int zsw, pzw, psf;  // z-strip column stride, staged window, CPML floats per ring slot
};

// slots of the shared-memory column ring: 4 columns in use by the stencils
// plus 4 in flight (deep prefetch for the latency-bound small grids)
constexpr int RING = 8;
constexpr int A2_TZ = TZ2;                             // pressure rows per block
constexpr int A2_THREADS = 128;                        // TZ + 3 velocity rows, one per thread
constexpr int A2_R8 = A2_TZ + 8;                       // p rows z0-4 .. z0+TZ+3
constexpr int A2_R4 = A2_TZ + 4;                       // velocity-input rows z0 .. z0+TZ+3
constexpr int A2_SLOT = A2_R8 + 4 * A2_R4 + A2_TZ;     // floats per ring slot
constexpr size_t A2_SMEM = 128 + sizeof(float) * (RING * A2_SLOT + 2 * RING * A2_R4);

// CPML floats per ring slot of the general kernel: two z-strip windows
// (dpdz, dvzdz) and the x-strip columns of dpdx and dvxdx
inline int a2_psi_floats(const Plan &p) {
  const bool zf = p.d.pml_faces & (GPI_ZMIN | GPI_ZMAX), xf = p.d.pml_faces & (GPI_XMIN | GPI_XMAX);
  return (zf ? 2 * p.pzw : 0) + (xf ? 2 * A2_TZ : 0);
}
inline size_t a2_smem_general(int psf) { return 128 + sizeof(float) * (RING * (A2_SLOT + psf) + 2 * RING * A2_R4); }

// MODE 0: interior tiles (no CPML, face or source: straight-line code);
// MODE 1: tiles away from the x edges and x strips (the band code over every
// column: z strips, z mirrors, sources); MODE 2: the same with x-strip
// columns; MODE 3: tiles with x-edge columns (the band code plus the general
// code for the edge and source columns).
template <int MODE>
__global__ void __launch_bounds__(A2_THREADS, MODE == 0 ? 6 : MODE == 1 ? 5 : 4) k_a2(const A2Args a) {
  constexpr bool FAST = MODE == 0, XPSI = MODE >= 2;
  constexpr int TZ = A2_TZ, R8 = A2_R8, R4 = A2_R4, SLOT = A2_SLOT;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  float *ring = reinterpret_cast<float *>(smem + 128);  // [RING][SLOT]: p | vx vz cx cz | dtK
  const int SL = FAST ? SLOT : SLOT + a.psf;            // floats per ring slot
  float *svx = ring + RING * SL;                         // [RING][R4] new velocities
  float *svz = svx + RING * R4;
  __shared__ int s_rng[3][2];
  __shared__ int s_err;
  const int t = threadIdx.x;
  const int4 tile = a.tiles[blockIdx.x];
  const int zb = tile.x, shot = tile.w;
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
  auto psA = [&](int i) -> const float * { return a.psA[i] + shot * a.pss[i]; };
  auto psB = [&](int i) -> float * { return a.psB[i] + shot * a.pss[i]; };
  auto slot = [&](int cc) -> int { return (cc - xbase) % RING; };
  // General kernel: the CPML memory of each column travels in its ring slot
  // (z-strip windows of dpdz and dvzdz, x-strip columns of dpdx and dvxdx).
  const int zt = FAST ? 0 : zstrip_touch(z0, TZ, nz, npml, zlo, zhi);
  const int zoff = FAST ? 0 : zstrip_off(zt, a.zsw, a.pzw);
  const int PZW = FAST ? 0 : a.pzw;
  // z strip indexed by strip slot (i: 0 dpdz, 1 dvzdz), x strip by row
  // (i: 0 dpdx, 1 dvxdx)
  auto PZ = [&](int i, int cc) -> const float * { return ring + slot(cc) * SL + SLOT + i * PZW - zoff; };
  auto PX = [&](int i, int cc) -> const float * { return ring + slot(cc) * SL + SLOT + 2 * PZW + i * TZ - z0; };
  // the same by ring slot
  auto PZs = [&](int i, int s) -> const float * { return ring + s * SL + SLOT + i * PZW - zoff; };
  auto PXs = [&](int i, int s) -> const float * { return ring + s * SL + SLOT + 2 * PZW + i * TZ - z0; };

  if (t == 0) {
    for (int s = 0; s < RING; s++) mbar_init(&bar[s], 4);  // one arrival per warp
    mbar_fence_init();
    s_err = 0;
  }
  if (t < 3) {
    const int kind = t == 0 ? 0 : t == 1 ? 2 : 3;
    const int g = shot * NKIND + kind;
    s_rng[t][0] = first_col(a.cells, a.gptr[g], a.gptr[g + 1], x0);
    s_rng[t][1] = a.gptr[g + 1];
  }
  __syncthreads();

  // producers: lane 0 of each warp issues its share of a column's bulk
  // copies and arrives on the slot's mbarrier with the bytes of its share
  // (warp 0 p, warp 1 vx vz, warp 2 cx and the dpdz CPML window, warp 3 cz
  // dtK and the dvzdz window; the x-strip CPML columns on warps 0 and 3)
  const int wq = t >> 5;
  const bool issuer = (t & 31) == 0;
  int next = xbase;
  auto issue = [&](int upto) {
    for (; next <= upto && next <= xlast; next++) {
      const int s = slot(next);
      float *sl = ring + s * SL;
      float *v = sl + R8, *pz = sl + SLOT, *px = pz + 2 * PZW;
      const int64_t oV = S(z0, next);
      int jx = -1;
      if constexpr (XPSI) {
        if (wq == 0) jx = pml_slot(next - 3, nx - 3, npml, xlo, xhi);
        if (wq == 3) jx = pml_slot(next, nx, npml, xlo, xhi);
      }
      uint32_t bytes = wq == 0 ? R8 * 4 : wq == 1 ? 2 * R4 * 4 : wq == 2 ? R4 * 4 : (R4 + TZ) * 4;
      if constexpr (!FAST) {
        if (zt && wq >= 2) bytes += PZW * 4;
        if (jx >= 0) bytes += TZ * 4;
      }
      mbar_expect_tx(&bar[s], bytes);
      if (wq == 0) {
        bulk_g2s(sl, a.pA + so + S(z0 - 4, next), R8 * 4, &bar[s]);
      } else if (wq == 1) {
        bulk_g2s(v + 0 * R4, a.vxA + so + oV, R4 * 4, &bar[s]);
        bulk_g2s(v + 1 * R4, a.vzA + so + oV, R4 * 4, &bar[s]);
      } else if (wq == 2) {
        bulk_g2s(v + 2 * R4, a.cx + oV, R4 * 4, &bar[s]);
      } else {
        bulk_g2s(v + 3 * R4, a.cz + oV, R4 * 4, &bar[s]);
        bulk_g2s(v + 4 * R4, a.dtK + oV, TZ * 4, &bar[s]);
      }
      if constexpr (!FAST) {
        if (zt && wq >= 2) bulk_g2s(pz + (wq - 2) * PZW, psA(wq == 2 ? 1 : 3) + ZS(next, zoff), PZW * 4, &bar[s]);
        if (jx >= 0) bulk_g2s(px + (wq == 0 ? 0 : TZ), psA(wq == 0 ? 0 : 2) + XS(jx, z0), TZ * 4, &bar[s]);
      }
    }
  };
  // interior and band tiles: each issuing lane keeps the source pointers of
  // its share of a column (at most three copies: fields advance by NZP per
  // column, z-strip CPML windows by zsw) and advances them per issue
  constexpr bool PROD = MODE <= 1;
  const float *fs0 = nullptr, *fs1 = nullptr, *fs2 = nullptr;
  int fd0 = 0, fd1 = 0, fd2 = 0, fst2 = NZP;
  uint32_t fn0 = 0, fn1 = 0, fn2 = 0;
  if constexpr (PROD) {
    const int64_t oV = S(z0, xbase);
    if (wq == 0) {
      fs0 = a.pA + so + S(z0 - 4, xbase), fd0 = 0, fn0 = R8 * 4;
    } else if (wq == 1) {
      fs0 = a.vxA + so + oV, fs1 = a.vzA + so + oV;
      fd0 = R8, fd1 = R8 + R4, fn0 = fn1 = R4 * 4;
    } else if (wq == 2) {
      fs0 = a.cx + oV, fd0 = R8 + 2 * R4, fn0 = R4 * 4;
    } else {
      fs0 = a.cz + oV, fs1 = a.dtK + oV;
      fd0 = R8 + 3 * R4, fd1 = R8 + 4 * R4, fn0 = R4 * 4, fn1 = TZ * 4;
    }
    if (!FAST && zt && wq >= 2) {
      // z-strip CPML windows: warp 2 dpdz, warp 3 dvzdz
      const float *pz = psA(wq == 2 ? 1 : 3) + ZS(xbase, zoff);
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
  auto wait_col = [&](int cc) {
    const int j = cc - xbase;
    if (!mbar_wait(&bar[j % RING], (j / RING) & 1)) s_err = 1;
  };

  InjCursor cvx, cvz, cst;
  cvx.init(a.cells, s_rng[0][0], s_rng[0][1]);
  cvz.init(a.cells, s_rng[1][0], s_rng[1][1]);
  cst.init(a.cells, s_rng[2][0], s_rng[2][1]);

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
  auto vel_fast = [&](int cc, int s3, int s2, int s1, int s0) {
    if (!vact) return;
    const int k = kq, kk = kq + 4;
    const float *pc = ring + s0 * SL, *v0 = pc + R8;
    const float vz = v0[R4 + k] + v0[3 * R4 + k] * (st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI);
    svz[s0 * R4 + k] = vz;
    if (kq < TZ) {
      const float *p3 = ring + s3 * SL, *p2 = ring + s2 * SL, *p1 = ring + s1 * SL;
      const float vx = v0[k] + v0[2 * R4 + k] * (st4(p3[kk], p2[kk], p1[kk], pc[kk]) * a.dxI);
      svx[s0 * R4 + k] = vx;
      if (cc < x1) {
        a.vxB[ov] = vx;
        a.vzB[ov] = vz;
      }
    }
  };
  // pressure of column c from velocity slots s0..s3 = columns c..c+3 (the
  // velocity half step: the old pressure, or nothing with vonly bit 2)
  auto str_fast = [&](int c, int s0, int s1, int s2, int s3) {
    if (t >= TZ) return;
    const int k = t;
    const float *pc = ring + s0 * SL;
    if (a.vonly) {
      if (!(a.vonly & 4)) a.pB[os] = pc[k + 4];
      return;
    }
    const float *w = svz + s0 * R4;
    const float Dx = st4(svx[s0 * R4 + k], svx[s1 * R4 + k], svx[s2 * R4 + k], svx[s3 * R4 + k]) * a.dxI;
    const float Dz = st4(w[k], w[k + 1], w[k + 2], w[k + 3]) * a.dzI;
    a.pB[os] = pc[k + 4] + (Dx + Dz) * pc[R8 + 4 * R4 + k];
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
    const int ncol = x1 - xbase;
    for (int base = 0; base < ncol; base += RING) {
      const uint32_t ph = (uint32_t)(base / RING) & 1u;
#pragma unroll
      for (int u = 0; u < RING; u++) {
        const int it = base + u;
        if (it >= ncol) break;
        const int c = xbase + it;
        if (!mbar_wait(&bar[(u + 3) % RING], ph ^ (uint32_t)((u + 3) / RING))) s_err = 1;
        vel_fast(c + 3, u % RING, (u + 1) % RING, (u + 2) % RING, (u + 3) % RING);
        __syncthreads();
        if (issuer && it >= 1 && c + RING - 1 <= xlast) issue_fast((u + RING - 1) % RING);
        if (c >= x0) str_fast(c, u % RING, (u + 1) % RING, (u + 2) % RING, (u + 3) % RING);
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
    // vz at row qq of column cc before its source (source of a mirror row)
    auto vz_any = [&](int qq, int cc) -> float {
      const int kv = qq - z0;
      const float *pc = ring + slot(cc) * SL, *v0 = pc + R8;
      float v = v0[R4 + kv];
      if (qq >= 4 && qq <= nz && cc >= 4 && cc <= nx - 3) {
        const int kk = kv + 4;
        float D = st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI;
        const int j = pml_slot(qq - 3, nz - 3, npml, zlo, zhi);
        if (j >= 0) D = cpml_p(D, 1, j, PZ(0, cc)[j], nullptr, false);
        v = v + v0[3 * R4 + kv] * D;
      }
      return v;
    };
    // Columns away from the x edges and from sources: every row in one
    // pass; rows outside an update domain keep their value, CPML terms where
    // a strip is met (psi staged in the ring slot of the column)
    // velocities of column cc from ring slots s3..s0 = columns cc-3..cc
    // (cells of the column's vx / vz sources in [ib0, ie0) / [ib1, ie1))
    auto vel_band = [&](int cc, int s3, int s2, int s1, int s0, int ib0, int ie0, int ib1, int ie1) {
      const int k = kqc, kk = kqc + 4, s = s0;
      const float *pc = ring + s * SL, *v0 = pc + R8;
      const float *p3 = ring + s3 * SL, *p2 = ring + s2 * SL, *p1s = ring + s1 * SL;
      const bool ownc = cc < x1;
      const bool ownx = ownc && ownr && q <= nz, ownz = ownc && ownr && q <= nz + 3;
      // branch-free: every row computes its derivatives; rows outside an
      // update domain keep their value, rows outside a strip their plain
      // derivative (selects)
      float Dz = st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI;
      float Dx = st4(p3[kk], p2[kk], p1s[kk], pc[kk]) * a.dxI;
      if (wzv) Dz = cpml_zs(Dz, cq1, PZs(0, s)[jq1c], jq1v >= 0, psB(1) + ZS(cc, jq1c), ownc && ownr);
      if constexpr (XPSI) {
        const int j0 = pml_slot(cc - 3, nx - 3, npml, xlo, xhi);
        if (j0 >= 0) Dx = cpml_xs(Dx, 0, j0, PXs(0, s)[q], vxr, psB(0) + XS(j0, q), ownx);
      }
      float vz = vzb ? v0[R4 + k] + v0[3 * R4 + k] * Dz : v0[R4 + k];
      float vx = vxr ? v0[k] + v0[2 * R4 + k] * Dx : v0[k];
      if (gany) {
        const float g = __shfl_sync(0xffffffffu, vz, glane);
        if (gsrc) vz = gok ? -g : -vz_any(gsrc, cc);
      }
      // add_velocity_source! (after the mirrors took their values)
      if (ib0 < ie0) inject(a.cells, a.amount, ib0, ie0, q, vx);
      if (ib1 < ie1) inject(a.cells, a.amount, ib1, ie1, q, vz);
      if (vact) svz[s * R4 + k] = vz;
      if (vact && kq < TZ) svx[s * R4 + k] = vx;
      const int64_t o = so + S(q, cc);
      if (ownz) a.vzB[o] = vz;
      if (ownx && kq < TZ) a.vxB[o] = vx;
    };
    // pressure of column c from velocity slots s0..s3 = columns c..c+3;
    // halo lanes recompute the last row and store nothing
    // (cells of the column's pressure sources in [bs, es))
    auto str_band = [&](int c, int s0, int s1, int s2, int s3, int bs, int es) {
      const int k = t < TZ ? t : TZ - 1, rk = z0 + k;
      const float *pc = ring + s0 * SL;
      float Dx = st4(svx[s0 * R4 + k], svx[s1 * R4 + k], svx[s2 * R4 + k], svx[s3 * R4 + k]) * a.dxI;
      const float *w = svz + s0 * R4;
      float Dz = st4(w[k], w[k + 1], w[k + 2], w[k + 3]) * a.dzI;
      if constexpr (XPSI) {
        const int j2 = pml_slot(c, nx, npml, xlo, xhi);
        if (j2 >= 0) Dx = cpml_xs(Dx, 2, j2, PXs(1, s0)[rk], srow, psB(2) + XS(j2, rk), true);
      }
      if (wzs) Dz = cpml_zs(Dz, cr3, PZs(1, s0)[jr3c], jr3v >= 0, psB(3) + ZS(c, jr3c), true);
      float pn = pc[k + 4] + (Dx + Dz) * pc[R8 + 4 * R4 + k];
      if (bs < es) inject(a.cells, a.amount, bs, es, r, pn);  // add_stress_source!
      if (srow) a.pB[so + S(r, c)] = pn;
    };
    if constexpr (MODE == 1) {
      // unrolled by RING: constant slot indices (see the interior loop)
      const int ncol = x1 - xbase;
      for (int base = 0; base < ncol; base += RING) {
        const uint32_t ph = (uint32_t)(base / RING) & 1u;
#pragma unroll
        for (int u = 0; u < RING; u++) {
          const int it = base + u;
          if (it >= ncol) break;
          const int c = xbase + it, cc = c + 3;
          int ib0, ie0, ib1, ie1, bs = 0, es = 0;
          cvx.range(a.cells, cc, ib0, ie0);
          cvz.range(a.cells, cc, ib1, ie1);
          if (c >= x0) cst.range(a.cells, c, bs, es);
          if (!mbar_wait(&bar[(u + 3) % RING], ph ^ (uint32_t)((u + 3) / RING))) s_err = 1;
          vel_band(cc, u % RING, (u + 1) % RING, (u + 2) % RING, (u + 3) % RING, ib0, ie0, ib1, ie1);
          __syncthreads();
          if (issuer && it >= 1 && c + RING - 1 <= xlast) issue_fast((u + RING - 1) % RING);
          if (c >= x0) str_band(c, u % RING, (u + 1) % RING, (u + 2) % RING, (u + 3) % RING, bs, es);
        }
      }
    } else if constexpr (MODE == 2) {
      // iteration it handles column c = xbase + it: slot(c + m) = (it + m) % RING
      const int ncol = x1 - xbase;
      for (int it = 0; it < ncol; it++) {
        const int c = xbase + it, cc = c + 3;
        int ib0, ie0, ib1, ie1, bs = 0, es = 0;
        cvx.range(a.cells, cc, ib0, ie0);
        cvz.range(a.cells, cc, ib1, ie1);
        if (c >= x0) cst.range(a.cells, c, bs, es);
        if (!mbar_wait(&bar[(it + 3) % RING], ((it + 3) / RING) & 1)) s_err = 1;
        vel_band(cc, it % RING, (it + 1) % RING, (it + 2) % RING, (it + 3) % RING, ib0, ie0, ib1, ie1);
        __syncthreads();
        if (issuer) issue(c + RING - 1);
        if (c >= x0) str_band(c, it % RING, (it + 1) % RING, (it + 2) % RING, (it + 3) % RING, bs, es);
      }
    } else {
      float vpre = 0.f;  // vx[r, nx] before its source (xmax mirror)
      auto vel_edge = [&](int cc, int ib0, int ie0, int ib1, int ie1) {
        if (!vact) return;
        const int k = kq, kk = kq + 4, s = slot(cc);
        const float *pc = ring + s * SL, *v0 = pc + R8;
        const bool ownc = cc >= x0 && (cc < x1 || lastx);
        if (kq < TZ) {
          const bool ownx = ownc && ownr && q <= nz;
          float vx;
          if (rxhi && cc >= nx + 2) {
            vx = cc == nx + 3 ? -vpre : -svx[slot(cc - 1) * R4 + k];  // vx[nx+3] = -vx[nx], vx[nx+2] = -vx[nx+1]
          } else {
            vx = v0[k];
            if (vxr && cc >= 4 && cc <= nx) {
              const float *p3 = ring + slot(cc - 3) * SL, *p2 = ring + slot(cc - 2) * SL,
                          *p1 = ring + slot(cc - 1) * SL;
              float D = st4(p3[kk], p2[kk], p1[kk], pc[kk]) * a.dxI;
              const int j0 = pml_slot(cc - 3, nx - 3, npml, xlo, xhi);
              if (j0 >= 0) D = cpml_p(D, 0, j0, PX(0, cc)[q], psB(0) + XS(j0, q), ownx);
              vx = vx + v0[2 * R4 + k] * D;
            }
            if (cc == nx) vpre = vx;
          }
          if (rxlo && cc == 4) {
            // dirichletxmin!: vx[1] = -vx[4] (before its source), vx[2] = -vx[3]
            const float g1 = -vx, g2 = -svx[slot(3) * R4 + k];
            svx[slot(1) * R4 + k] = g1;
            svx[slot(2) * R4 + k] = g2;
            if (x0 == 1 && ownr && q <= nz) {
              a.vxB[so + S(q, 1)] = g1;
              a.vxB[so + S(q, 2)] = g2;
            }
          }
          if (vsrc) inject(a.cells, a.amount, ib0, ie0, q, vx);
          svx[s * R4 + k] = vx;
          if (ownx) a.vxB[so + S(q, cc)] = vx;
        }
        float vz;
        if (gsrc) {
          vz = -vz_any(gsrc, cc);  // dirichletzmin!/zmax!
        } else {
          vz = v0[R4 + k];
          if (vzr && cc >= 4 && cc <= nx - 3) {
            float D = st4(pc[kk - 3], pc[kk - 2], pc[kk - 1], pc[kk]) * a.dzI;
            if (jq1 >= 0) D = cpml_z(D, cq1, PZ(0, cc)[jq1], psB(1) + ZS(cc, jq1), ownc && ownr && cc <= nx);
            vz = vz + v0[3 * R4 + k] * D;
          }
        }
        if (vsrc) inject(a.cells, a.amount, ib1, ie1, q, vz);
        svz[s * R4 + k] = vz;
        if (ownc && ownr && cc <= nx && q <= nz + 3) a.vzB[so + S(q, cc)] = vz;
      };
      auto str_edge = [&](int c, int bs, int es) {
        if (!srow) return;
        const int k = t;
        const float *pc = ring + slot(c) * SL;
        float pn = pc[k + 4];
        if (!a.vonly) {
          float Dx = st4(svx[slot(c) * R4 + k], svx[slot(c + 1) * R4 + k], svx[slot(c + 2) * R4 + k],
                         svx[slot(c + 3) * R4 + k]) * a.dxI;
          const int j2 = pml_slot(c, nx, npml, xlo, xhi);
          if (j2 >= 0) Dx = cpml_p(Dx, 2, j2, PX(1, c)[r], psB(2) + XS(j2, r), true);
          const float *w = svz + slot(c) * R4;
          float Dz = st4(w[k], w[k + 1], w[k + 2], w[k + 3]) * a.dzI;
          if (jr3 >= 0) Dz = cpml_z(Dz, cr3, PZ(1, c)[jr3], psB(3) + ZS(c, jr3), true);
          pn = pn + (Dx + Dz) * pc[R8 + 4 * R4 + k];
          inject(a.cells, a.amount, bs, es, r, pn);  // add_stress_source!
        }
        if (!(a.vonly & 4)) a.pB[so + S(r, c)] = pn;
      };
      // one sweep: iterations c < x0 only compute the first velocity columns
      for (int c = x0 - 3; c < x1; c++) {
        const int cc = c + 3;
        int ib0, ie0, ib1, ie1, bs = 0, es = 0;
        cvx.range(a.cells, cc, ib0, ie0);
        cvz.range(a.cells, cc, ib1, ie1);
        if (c >= x0) cst.range(a.cells, c, bs, es);
        // general code for x edges, mirrors and sources (block-uniform);
        // otherwise the band code over every row
        const bool gv = colfull_v(cc) || ib0 < ie0 || ib1 < ie1;
        const bool gs = colfull_s(c) || bs < es;
        wait_col(cc);
        if (gv)
          vel_edge(cc, ib0, ie0, ib1, ie1);
        else
          vel_band(cc, slot(cc - 3), slot(cc - 2), slot(cc - 1), slot(cc), ib0, ie0, ib1, ie1);
        __syncthreads();
        if (issuer) issue(c + RING - 1);
        if (c >= x0) {
          if (gs)
            str_edge(c, bs, es);
          else
            str_band(c, slot(c), slot(c + 1), slot(c + 2), slot(c + 3), bs, es);
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

int step_acoustic2d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  if (mode == GPI_ADJOINT && !vonly) return step_adjoint_acoustic2d(p, it);
  (void)ipw_mask;
  (void)it;
  return step_a2_wavefield(p, 0, vonly);
}

// one time step of wavefield ipw (0 the modelled, 1 the adjoint wavefield)
int step_a2_wavefield(Plan *p, int ipw, int vonly) {
  A2Args a;
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
  const int A = p->cur[ipw], B = A ^ 1;
  a.pA = p->state[A][ipw][GPI_P];
  a.vxA = p->state[A][ipw][GPI_VX];
  a.vzA = p->state[A][ipw][GPI_VZ];
  a.pB = p->state[B][ipw][GPI_P];
  a.vxB = p->state[B][ipw][GPI_VX];
  a.vzB = p->state[B][ipw][GPI_VZ];
  for (int q = 0; q < 4; q++) {
    a.psA[q] = p->psi[A][ipw][q];
    a.psB[q] = p->psi[B][ipw][q];
    a.pss[q] = p->psi_stride[q];
  }
  a.cx = p->coef[0];
  a.cz = p->coef[1];
  a.dtK = p->coef[2];
  a.pml = p->pml;
  a.cells = p->d_cells;
  a.gptr = p->d_group_ptr + (int64_t)ipw * p->d.nshots * NKIND;  // this wavefield's cell groups
  a.amount = p->d_amount;
  a.vonly = vonly;
  a.err = p->d_err;
  a.tiles = p->d_tiles;
  a.zsw = p->zsw;
  a.pzw = p->pzw;
  // shared memory per block: the ring with the CPML memory each mode stages
  const bool zf = p->d.pml_faces & (GPI_ZMIN | GPI_ZMAX);
  const int psf[4] = {0, zf ? 2 * p->pzw : 0, a2_psi_floats(*p), a2_psi_floats(*p)};
  size_t smem[4];
  for (int m = 0; m < 4; m++) smem[m] = m == 0 ? A2_SMEM : a2_smem_general(psf[m]);
  void (*const fn[4])(A2Args) = {k_a2<0>, k_a2<1>, k_a2<2>, k_a2<3>};
  for (int m = 0; m < 4; m++)
    if (int rc = ensure_smem_attr(p, (const void *)fn[m], 0 + m, smem[m])) return rc;
  auto launch = [&](int m, int first, int n, cudaStream_t st) {
    if (n <= 0) return;
    A2Args g = a;
    g.tiles = p->d_tiles + first;
    g.psf = psf[m];
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
  p->cur[ipw] ^= 1;
  return GPI_OK;
}

}  // namespace gpi
