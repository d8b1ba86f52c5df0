// k_elastic2d.cu -- fused 2-D elastic (P-SV) time step (order 4).
//
// One launch advances every shot by one time step:
//   compute_dstress! + memory*! + compute_v! + dirichlet*! + velocity sources
//   compute_dv! + memory*! + compute_stressii!/ij! + free surface + stress sources
// (src/fdtd/advance_elastic.jl:10-230, :534-682, src/fdtd/cpml.jl:158-215,
//  src/fdtd/dirichlet.jl:1-79, src/fdtd/source.jl:79-97, :124-177).
// Reference index arithmetic (h = 3, shapes from src/fields.jl:277-671):
//   vx[r, c]  -= cx (D_x txx[r, c-3..c]   + D_z txz[r-3..r, c-3]),  r 4..nz-3, c 4..nx
//   vz[q, c]  -= cz (D_x txz[q-3, c-3..c] + D_z tzz[q-3..q, c]),    q 4..nz,   c 4..nx-3
//   txx[r, c] -= dtM D_x vx[r, c..c+3] + dtl D_z vz[r..r+3, c]            (all cells)
//   tzz[r, c] -= dtM D_z vz[r..r+3, c] + dtl D_x vx[r, c..c+3]
//   txz[r, c] -= mu (D_z vx[r..r+3, c+3] + D_x vz[r+3, c..c+3]),  r <= nz-3, c <= nx-3
//
// Work decomposition.  A block owns TZ rows x L columns of the normal-stress
// grid of one shot and sweeps its columns.  For every column it needs ten
// input columns (three stresses over rows z0-4..z0+TZ+3, the two old
// velocities and their coefficients over z0..z0+TZ+3, dtM, dtl, mu over
// z0..z0+TZ-1); one producer thread streams them into an 8-column ring in
// shared memory with bulk asynchronous copies (cp.async.bulk, the TMA
// engine) that complete on one mbarrier per ring slot, four columns ahead
// of the compute.  TZ threads (plus 3 of an extra warp for the halo rows)
// compute from shared memory only.  Halo velocities (3 columns right of and
// 3 rows below the tile) are recomputed from the input buffer, so the state
// is ping-ponged and a time step is one pass over HBM: 10 arrays read,
// 5 written, 60 B per cell update.
#include "k_stencil.cuh"

namespace gpi {

struct E2Args {
  int nz, nx, NZP;
  int64_t fs;
  int npml, faces, rigid, free;
  float dxI, dzI;
  int nzb;
  const float *txxA, *tzzA, *txzA, *vxA, *vzA;
  float *txxB, *tzzB, *txzB, *vxB, *vzB;
  const float *psA[8];
  float *psB[8];
  int64_t pss[8];
  const float *cx, *cz, *mu, *dtM, *dtl;
  const float *pml;  // [8][3][2*npml]
  const InjCell *cells;
  const int32_t *gptr;
  const float *amount;
  int vonly;
  int *err;  // set when a pipeline wait gives up
  const int4 *tiles;  // (z-block, first column, end column, shot) per block
  int zsw, pzw, psf;  // z-strip column stride, staged window, CPML floats per ring slot
};

// slots of the shared-memory column ring: 4 columns in use by the stencils
// plus 2 in flight; 6 keeps an interior block at 37 KB (6 blocks per SM).
// The band tiles take 5 (one column in flight) so that six of their blocks
// fit an SM as well (80 registers, about 35 KB)
constexpr int RING = 6;
__host__ __device__ constexpr int e2_ring(int mode) { return mode == 1 ? 5 : RING; }
constexpr int E2_TZ = TZ2;                                      // stress rows per block
constexpr int E2_THREADS = 128;                                 // TZ + 3 velocity rows, one per thread
constexpr int E2_R8 = E2_TZ + 8;                                // stress rows z0-4 .. z0+TZ+3
constexpr int E2_R4 = E2_TZ + 4;                                // velocity-input rows z0 .. z0+TZ+3
constexpr int E2_SLOT = 3 * E2_R8 + 4 * E2_R4 + 3 * E2_TZ;      // floats per ring slot
constexpr size_t E2_SMEM = 128 + sizeof(float) * (RING * E2_SLOT + 2 * RING * E2_R4);

// CPML floats per ring slot of the general kernel: four z-strip windows
// (derivatives 2, 3, 5, 6) and the x-strip columns of derivatives 0, 1
// (velocity rows) and 4, 7 (stress rows)
inline int e2_psi_floats(const Plan &p) {
  const bool zf = p.d.pml_faces & (GPI_ZMIN | GPI_ZMAX), xf = p.d.pml_faces & (GPI_XMIN | GPI_XMAX);
  return (zf ? 4 * p.pzw : 0) + (xf ? 2 * E2_R4 + 2 * E2_TZ : 0);
}
inline size_t e2_smem_general(int psf, int ring) {
  return 128 + sizeof(float) * (ring * (E2_SLOT + psf) + 2 * ring * E2_R4);
}

// MODE 0: interior tiles (no CPML, face or source: straight-line code);
// MODE 1: tiles away from the x edges and x strips (the band code over every
// column: z strips, z mirrors, the free surface, sources); MODE 2: the same
// with x-strip columns; MODE 3: tiles with x-edge columns (the band code plus
// the general code for the edge and source columns).
// The body takes the arguments by reference: the kernel's own parameters
// (one plan) or a plan's arguments copied to shared memory (k_e2_batch).
template <int MODE>
__device__ __forceinline__ void e2_body(const E2Args &a, const int4 tile) {
  constexpr bool FAST = MODE == 0, XPSI = MODE >= 2;
  constexpr int RING = e2_ring(MODE);
  constexpr int TZ = E2_TZ, R8 = E2_R8, R4 = E2_R4, SLOT = E2_SLOT;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);  // one mbarrier per ring slot
  float *ring = reinterpret_cast<float *>(smem + 128);  // [RING][SLOT]
  const int SL = FAST ? SLOT : SLOT + a.psf;            // floats per ring slot
  float *svx = ring + RING * SL;                         // [RING][R4] new velocities
  float *svz = svx + RING * R4;
  __shared__ int s_rng[3][2];
  __shared__ int s_err;
  const int t = threadIdx.x;
  const int zb = tile.x, shot = tile.w & 0xffff;  // (the high half: a batch's plan slot)
  const int z0 = 1 + zb * TZ, x0 = tile.y, x1 = tile.z;
  const int xbase = x0 - 3, xlast = x1 + 2;  // input columns of this block
  const bool lastx = x1 == a.nx + 1, lastz = zb == a.nzb - 1;
  const int nz = a.nz, nx = a.nx, npml = a.npml, NZP = a.NZP;
  const int64_t so = (int64_t)shot * a.fs;
  const bool xlo = a.faces & GPI_XMIN, xhi = a.faces & GPI_XMAX, zlo = a.faces & GPI_ZMIN, zhi = a.faces & GPI_ZMAX;
  const bool rxlo = a.rigid & GPI_XMIN, rxhi = a.rigid & GPI_XMAX, rzlo = a.rigid & GPI_ZMIN, rzhi = a.rigid & GPI_ZMAX;
  const bool fsurf = a.free & GPI_ZMIN;
  const int P6 = 6 * npml;  // floats per derivative field in a.pml
  auto S = [&](int rr, int cc) -> int64_t { return (int64_t)(cc + XOFF - 1) * NZP + (rr + ZOFF - 1); };
  auto XS = [&](int j, int rr) -> int64_t { return (int64_t)j * NZP + (rr + ZOFF - 1); };       // x strip
  auto ZS = [&](int cc, int j) -> int64_t { return (int64_t)(cc + XOFF - 1) * a.zsw + j; };  // z strip
  auto psA = [&](int q) -> const float * { return a.psA[q] + shot * a.pss[q]; };
  auto psB = [&](int q) -> float * { return a.psB[q] + shot * a.pss[q]; };
  // General kernel: the CPML memory of each column travels in its ring slot
  // (z-strip windows of derivatives 2, 3, 5, 6 and x-strip columns of
  // derivatives 0, 1, 4, 7), so no thread waits on a global load.
  const int zt = FAST ? 0 : zstrip_touch(z0, TZ, nz, npml, zlo, zhi);
  const int zoff = FAST ? 0 : zstrip_off(zt, a.zsw, a.pzw);
  const int PZW = FAST ? 0 : a.pzw;
  // ring views of input column cc
  auto slot = [&](int cc) -> int { return (cc - xbase) % RING; };
  auto T = [&](int f, int cc) -> const float * { return ring + slot(cc) * SL + f * R8; };           // txx tzz txz
  auto V = [&](int f, int cc) -> const float * { return ring + slot(cc) * SL + 3 * R8 + f * R4; };  // vx vz cx cz
  auto C = [&](int f, int cc) -> const float * {
    return ring + slot(cc) * SL + 3 * R8 + 4 * R4 + f * TZ;  // dtM dtl mu
  };
  // staged CPML memory of column cc: z strip indexed by strip slot
  // (i: 0 dtauzzdz, 1 dtauxzdz, 2 dvzdz, 3 dvxdz), x strip by row (i: 0
  // dtauxxdx, 1 dtauxzdx over velocity rows, 2 dvxdx, 3 dvzdx over stress rows)
  auto PZ = [&](int i, int cc) -> const float * { return ring + slot(cc) * SL + SLOT + i * PZW - zoff; };
  auto PX = [&](int i, int cc) -> const float * {
    return ring + slot(cc) * SL + SLOT + 4 * PZW + (i < 2 ? i * R4 : 2 * R4 + (i - 2) * TZ) - z0;
  };
  // the same by ring slot
  auto PZs = [&](int i, int s) -> const float * { return ring + s * SL + SLOT + i * PZW - zoff; };
  auto PXs = [&](int i, int s) -> const float * {
    return ring + s * SL + SLOT + 4 * PZW + (i < 2 ? i * R4 : 2 * R4 + (i - 2) * TZ) - z0;
  };

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

  // ---- producers: lane 0 of each warp issues its share of a column's bulk
  // copies and arrives on the slot's mbarrier with the bytes of its share
  // (warp 0 the stresses, warp 1 vx vz cx, warp 2 cz dtM, warp 3 dtl mu; in
  // the general kernel also the CPML memory, spread the same way) ----
  const int wq = t >> 5;
  const bool issuer = (t & 31) == 0;
  int next = xbase;
  auto issue = [&](int upto) {
    for (; next <= upto && next <= xlast; next++) {
      const int s = slot(next);
      float *sl = ring + s * SL;
      const int64_t oT = so + S(z0 - 4, next), oV = S(z0, next);
      float *v = sl + 3 * R8, *cf = v + 4 * R4;
      float *pz = sl + SLOT, *px = pz + 4 * PZW;
      int jx = -1;
      if constexpr (XPSI) {
        jx = wq == 0 ? pml_slot(next - 3, nx - 3, npml, xlo, xhi)
           : wq == 1 ? pml_slot(next - 3, nx - 6, npml, xlo, xhi)
           : wq == 2 ? pml_slot(next, nx, npml, xlo, xhi)
                     : pml_slot(next, nx - 3, npml, xlo, xhi);
      }
      const int jrows = wq < 2 ? R4 : TZ;  // x-strip CPML rows of this warp's derivative
      uint32_t bytes = wq == 0 ? 3 * R8 * 4 : wq == 1 ? 3 * R4 * 4 : wq == 2 ? (R4 + TZ) * 4 : 2 * TZ * 4;
      if constexpr (!FAST) {
        if (zt && wq >= 2) bytes += 2 * PZW * 4;
        if (jx >= 0) bytes += jrows * 4;
      }
      mbar_expect_tx(&bar[s], bytes);
      if (wq == 0) {
        bulk_g2s(sl + 0 * R8, a.txxA + oT, R8 * 4, &bar[s]);
        bulk_g2s(sl + 1 * R8, a.tzzA + oT, R8 * 4, &bar[s]);
        bulk_g2s(sl + 2 * R8, a.txzA + oT, R8 * 4, &bar[s]);
      } else if (wq == 1) {
        bulk_g2s(v + 0 * R4, a.vxA + so + oV, R4 * 4, &bar[s]);
        bulk_g2s(v + 1 * R4, a.vzA + so + oV, R4 * 4, &bar[s]);
        bulk_g2s(v + 2 * R4, a.cx + oV, R4 * 4, &bar[s]);
      } else if (wq == 2) {
        bulk_g2s(v + 3 * R4, a.cz + oV, R4 * 4, &bar[s]);
        bulk_g2s(cf + 0 * TZ, a.dtM + oV, TZ * 4, &bar[s]);
      } else {
        bulk_g2s(cf + 1 * TZ, a.dtl + oV, TZ * 4, &bar[s]);
        bulk_g2s(cf + 2 * TZ, a.mu + oV, TZ * 4, &bar[s]);
      }
      if constexpr (!FAST) {
        if (zt && wq >= 2) {
          // z-strip windows: warp 2 derivatives 2 3, warp 3 derivatives 5 6
          const int64_t oz = ZS(next, zoff);
          const int i0 = wq == 2 ? 0 : 2;
          bulk_g2s(pz + i0 * PZW, psA(wq == 2 ? 2 : 5) + oz, PZW * 4, &bar[s]);
          bulk_g2s(pz + (i0 + 1) * PZW, psA(wq == 2 ? 3 : 6) + oz, PZW * 4, &bar[s]);
        }
        if (jx >= 0) {
          // x-strip column of derivative 0, 1, 4 or 7
          const int q8 = wq == 0 ? 0 : wq == 1 ? 1 : wq == 2 ? 4 : 7;
          float *dst = px + (wq < 2 ? wq * R4 : 2 * R4 + (wq - 2) * TZ);
          bulk_g2s(dst, psA(q8) + XS(jx, z0), jrows * 4, &bar[s]);
        }
      }
    }
  };
  // interior and band tiles: each issuing lane keeps the source pointers of
  // its share of a column (at most four copies: fields advance by NZP per
  // column, z-strip CPML windows by zsw) and advances them per issue, so the
  // steady-state producer work is a few instructions
  constexpr bool PROD = MODE <= 1;
  const float *fs0 = nullptr, *fs1 = nullptr, *fs2 = nullptr, *fs3 = nullptr;
  int fd0 = 0, fd1 = 0, fd2 = 0, fd3 = 0, fst2 = NZP, fst3 = NZP;
  uint32_t fn0 = 0, fn1 = 0, fn2 = 0, fn3 = 0;
  if constexpr (PROD) {
    const int64_t oT = so + S(z0 - 4, xbase), oV = S(z0, xbase);
    if (wq == 0) {
      fs0 = a.txxA + oT, fs1 = a.tzzA + oT, fs2 = a.txzA + oT;
      fd0 = 0, fd1 = R8, fd2 = 2 * R8;
      fn0 = fn1 = fn2 = R8 * 4;
    } else if (wq == 1) {
      fs0 = a.vxA + so + oV, fs1 = a.vzA + so + oV, fs2 = a.cx + oV;
      fd0 = 3 * R8, fd1 = 3 * R8 + R4, fd2 = 3 * R8 + 2 * R4;
      fn0 = fn1 = fn2 = R4 * 4;
    } else if (wq == 2) {
      fs0 = a.cz + oV, fs1 = a.dtM + oV;
      fd0 = 3 * R8 + 3 * R4, fd1 = 3 * R8 + 4 * R4;
      fn0 = R4 * 4, fn1 = TZ * 4;
    } else {
      fs0 = a.dtl + oV, fs1 = a.mu + oV;
      fd0 = 3 * R8 + 4 * R4 + TZ, fd1 = 3 * R8 + 4 * R4 + 2 * TZ;
      fn0 = fn1 = TZ * 4;
    }
    if (!FAST && zt && wq >= 2) {
      // z-strip CPML windows: warp 2 derivatives 2 3, warp 3 derivatives 5 6
      const int64_t oz = ZS(xbase, zoff);
      const int i0 = wq == 2 ? 0 : 2;
      fs2 = psA(wq == 2 ? 2 : 5) + oz, fs3 = psA(wq == 2 ? 3 : 6) + oz;
      fd2 = SLOT + i0 * PZW, fd3 = SLOT + (i0 + 1) * PZW;
      fn2 = fn3 = PZW * 4;
      fst2 = fst3 = a.zsw;
    }
  }
  // the next column of this warp's share into ring slot sl
  auto issue_fast = [&](int sl) {
    float *d = ring + sl * SL;
    mbar_expect_tx(&bar[sl], fn0 + fn1 + fn2 + fn3);
    bulk_g2s(d + fd0, fs0, fn0, &bar[sl]);
    bulk_g2s(d + fd1, fs1, fn1, &bar[sl]);
    if (fn2) bulk_g2s(d + fd2, fs2, fn2, &bar[sl]);
    if (fn3) bulk_g2s(d + fd3, fs3, fn3, &bar[sl]);
    fs0 += NZP, fs1 += NZP, fs2 += fst2, fs3 += fst3;
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

  // this thread's velocity row: t < TZ -> z0+t, halo lanes -> z0+TZ+0..2
  const int kq = t < TZ + 3 ? t : -1;
  const int q = z0 + kq;
  const bool vact = kq >= 0;
  const bool ownr = kq >= 0 && (kq < TZ || lastz);

  // ---- per-thread row constants: velocity row q, stress row r ----
  const bool vxr = q >= 4 && q <= nz - 3, vzr = q >= 4 && q <= nz;
  const int jq3 = pml_slot(q - 3, nz - 6, npml, zlo, zhi);  // dtauxzdz (z strip)
  const int jq2 = pml_slot(q - 3, nz - 3, npml, zlo, zhi);  // dtauzzdz (z strip)
  // vz mirror source of a ghost row (dirichletzmin!/zmax!), 0 otherwise;
  // rows below nz+3 are never stored nor read
  const int gsrc = (rzlo && q <= 2) ? 5 - q : (rzhi && q >= nz + 2 && q <= nz + 3) ? 2 * nz + 3 - q : 0;
  const int r = z0 + t;
  const bool srow = t < TZ && r <= nz;
  const int jr5 = pml_slot(r, nz, npml, zlo, zhi);      // dvzdz (z strip)
  const int jr6 = pml_slot(r, nz - 3, npml, zlo, zhi);  // dvxdz (z strip)
  const bool xzrow = r <= nz - 3;
  const bool fsrow = fsurf && r == 1;

  // CPML: psi' = b psi + a D ; D' = D kI + psi'  (profile [a | b | kI])
  auto cpml_p = [&](float D, int q8, int j, float psi_old, float *dst, bool own) -> float {
    const float *cf = a.pml + q8 * P6;
    const float psi = __ldg(cf + 2 * npml + j) * psi_old + __ldg(cf + j) * D;
    if (own) *dst = psi;
    return D * __ldg(cf + 4 * npml + j) + psi;
  };
  // the z-strip profile of this thread's rows, loaded once
  auto zprof = [&](int q8, int j) -> float3 {
    if (FAST || j < 0) return make_float3(0.f, 0.f, 0.f);
    const float *cf = a.pml + q8 * P6;
    return make_float3(__ldg(cf + j), __ldg(cf + 2 * npml + j), __ldg(cf + 4 * npml + j));
  };
  const float3 cq2 = zprof(2, jq2), cq3 = zprof(3, jq3), cr5 = zprof(5, jr5), cr6 = zprof(6, jr6);
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
  auto cpml_xs = [&](float D, int q8, int j, float psi_old, bool on, float *dst, bool own) -> float {
    const float *cf = a.pml + q8 * P6;
    const float psi = __ldg(cf + 2 * npml + j) * psi_old + __ldg(cf + j) * D;
    if (on && own) *dst = psi;
    return on ? D * __ldg(cf + 4 * npml + j) + psi : D;
  };
  // vz at row qq of column cc before its source (source of a mirror row)
  auto vz_any = [&](int qq, int cc) -> float {
    const int kv = qq - z0;
    float v = V(1, cc)[kv];
    if (qq >= 4 && qq <= nz && cc >= 4 && cc <= nx - 3) {
      const int k = qq - z0 + 4;
      float Dx = st4(T(2, cc - 3)[k - 3], T(2, cc - 2)[k - 3], T(2, cc - 1)[k - 3], T(2, cc)[k - 3]) * a.dxI;
      int j = pml_slot(cc - 3, nx - 6, npml, xlo, xhi);
      if (j >= 0) Dx = cpml_p(Dx, 1, j, PX(1, cc)[qq], nullptr, false);
      const float *zz = T(1, cc);
      float Dz = st4(zz[k - 3], zz[k - 2], zz[k - 1], zz[k]) * a.dzI;
      j = pml_slot(qq - 3, nz - 3, npml, zlo, zhi);
      if (j >= 0) Dz = cpml_p(Dz, 2, j, PZ(0, cc)[j], nullptr, false);
      v = v - V(3, cc)[kv] * (Dx + Dz);
    }
    return v;
  };
  // tzz at row 2 of column c before its source (free_surface_mirror!)
  auto tzz_row2 = [&](int c) -> float {
    const int kk = 1;
    const float *u0 = svx + slot(c) * R4, *u1 = svx + slot(c + 1) * R4, *u2 = svx + slot(c + 2) * R4,
                *u3 = svx + slot(c + 3) * R4, *w = svz + slot(c) * R4;
    float dvxdx = st4(u0[kk], u1[kk], u2[kk], u3[kk]) * a.dxI;
    int j = pml_slot(c, nx, npml, xlo, xhi);
    if (j >= 0) dvxdx = cpml_p(dvxdx, 4, j, PX(2, c)[2], nullptr, false);
    float dvzdz = st4(w[kk], w[kk + 1], w[kk + 2], w[kk + 3]) * a.dzI;
    j = pml_slot(2, nz, npml, zlo, zhi);
    if (j >= 0) dvzdz = cpml_p(dvzdz, 5, j, PZ(2, c)[j], nullptr, false);
    return T(1, c)[kk + 4] - (C(0, c)[kk] * dvzdz) - (C(1, c)[kk] * (dvxdx));
  };
  float vpre = 0.f;  // vx[q, nx] before its source (xmax mirror)
  // ---- prologue: stresses of columns x0-3 .. x0-1 ----
  for (int cc = xbase; cc < x0 && cc <= xlast; cc++) wait_col(cc);

  // the interior code: every row inside every update domain, no CPML, no
  // face, no source
  // global addresses of this thread's rows, advanced one column per
  // iteration: velocities of column xbase+3+it, stresses of column xbase+it
  int64_t ov = so + S(q, xbase + 3), os = so + S(z0 + t, xbase);
  // velocities of column cc from ring slots s3..s0 = columns cc-3..cc
  auto vel_fast = [&](int cc, int s3, int s2, int s1, int s0) {
    if (!vact) return;
    const int k = kq, kk = kq + 4;
    const float *b3 = ring + s3 * SL, *b2 = ring + s2 * SL, *b1 = ring + s1 * SL, *b0 = ring + s0 * SL;
    const float *v0 = b0 + 3 * R8, *z3 = b3 + 2 * R8, *zz = b0 + R8;
    const float Dx = st4(b3[kk], b2[kk], b1[kk], b0[kk]) * a.dxI;
    const float Dz = st4(z3[kk - 3], z3[kk - 2], z3[kk - 1], z3[kk]) * a.dzI;
    const float vx = v0[k] - v0[2 * R4 + k] * (Dx + Dz);
    const float Dx2 = st4(z3[kk - 3], b2[2 * R8 + kk - 3], b1[2 * R8 + kk - 3], b0[2 * R8 + kk - 3]) * a.dxI;
    const float Dz2 = st4(zz[kk - 3], zz[kk - 2], zz[kk - 1], zz[kk]) * a.dzI;
    const float vz = v0[R4 + k] - v0[3 * R4 + k] * (Dx2 + Dz2);
    svx[s0 * R4 + k] = vx;
    svz[s0 * R4 + k] = vz;
    if (cc < x1 && kq < TZ) {
      a.vxB[ov] = vx;
      a.vzB[ov] = vz;
    }
  };
  // stresses of column c from velocity slots s0..s3 = columns c..c+3
  auto str_fast = [&](int c, int s0, int s1, int s2, int s3) {
    if (t >= TZ) return;
    const int k = t;
    const float *u0 = svx + s0 * R4, *u1 = svx + s1 * R4, *u2 = svx + s2 * R4, *u3 = svx + s3 * R4;
    const float *w0 = svz + s0 * R4, *w1 = svz + s1 * R4, *w2 = svz + s2 * R4, *w3 = svz + s3 * R4;
    const float *bc = ring + s0 * SL, *cf = bc + 3 * R8 + 4 * R4;
    const float dvxdx = st4(u0[k], u1[k], u2[k], u3[k]) * a.dxI;
    const float dvzdz = st4(w0[k], w0[k + 1], w0[k + 2], w0[k + 3]) * a.dzI;
    const float M = cf[k], Lm = cf[TZ + k], mu = cf[2 * TZ + k];
    const float txx = bc[k + 4] - (M * dvxdx) - (Lm * (dvzdz));
    const float tzz = bc[R8 + k + 4] - (M * dvzdz) - (Lm * (dvxdx));
    const float dvxdz = st4(u3[k], u3[k + 1], u3[k + 2], u3[k + 3]) * a.dzI;
    const float dvzdx = st4(w0[k + 3], w1[k + 3], w2[k + 3], w3[k + 3]) * a.dxI;
    const float txz = bc[2 * R8 + k + 4] - mu * (dvxdz + dvzdx);
    a.txxB[os] = txx;
    a.tzzB[os] = tzz;
    a.txzB[os] = txz;
  };

  // Dispatch per warp and per column: a warp runs the straight-line code
  // unless one of its rows or the current column touches a CPML strip, a
  // rigid or free face, a domain edge or a source cell.
  if constexpr (FAST) {
    // interior tile: inside every update domain, no CPML, no face, no
    // source.
    // iteration it handles column c = xbase + it: slot(c + m) = (it + m) %
    // RING.  The loop is unrolled by RING so that every slot index is a
    // constant (base is a multiple of RING; the parity of a slot's mbarrier
    // flips once per RING columns)
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
  auto colfull_s = [&](int c) { return a.vonly || c <= 1 || c >= nx - 4; };
  // per-row constants of the band path: the row inside each update domain,
  // the CPML slots only where the row is updated
  const int kqc = vact ? kq : 0;
  const bool vxb = vact && vxr, vzb = vact && vzr;
  const int jq3v = vxb ? jq3 : -1, jq2v = vzb ? jq2 : -1;
  const int jr5v = srow ? jr5 : -1, jr6v = (srow && xzrow) ? jr6 : -1;
  // in-window strip slots to read when a row is outside its strip
  const int jq3c = jq3v >= 0 ? jq3v : zoff, jq2c = jq2v >= 0 ? jq2v : zoff;
  const int jr5c = jr5v >= 0 ? jr5v : zoff, jr6c = jr6v >= 0 ? jr6v : zoff;
  // warps with a z-strip row (velocity / stress rows): the others skip the
  // memory-variable code as a whole
  const bool wzv = __any_sync(0xffffffffu, jq3v >= 0 || jq2v >= 0);
  const bool wzs = __any_sync(0xffffffffu, jr5v >= 0 || jr6v >= 0);
  // ghost rows of vz (dirichletzmin!/zmax!) read their mirror source from
  // the lane that computes it, when that lane is in the same warp
  const int lane = t & 31;
  const int gdl = gsrc ? gsrc - q : 0;
  const bool gok = lane + gdl >= 0 && lane + gdl < 32;
  const int glane = gok ? lane + gdl : lane;
  const bool gany = __any_sync(0xffffffffu, gsrc != 0);
  const bool fsblk = fsurf && z0 == 1;  // the free-surface row is lane 0 of warp 0
  {
    // Columns away from the x edges and from sources: every row in one
    // pass; rows outside an update domain keep their value, CPML terms where
    // a strip is met (psi staged in the ring slot of the column)
    // velocities of column cc from ring slots s3..s0 = columns cc-3..cc
    // (cells of the column's vx / vz sources in [ib0, ie0) / [ib1, ie1))
    auto vel_band = [&](int cc, int s3, int s2, int s1, int s0, int ib0, int ie0, int ib1, int ie1) {
      const int k = kqc, kk = kqc + 4, s = s0;
      const bool ownc = cc < x1;
      const bool ownx = ownc && ownr && q <= nz, ownz = ownc && ownr && q <= nz + 3;
      const float *b3 = ring + s3 * SL, *b2 = ring + s2 * SL, *b1 = ring + s1 * SL, *b0 = ring + s * SL;
      const float *v0 = b0 + 3 * R8, *z3 = b3 + 2 * R8, *zz = b0 + R8;
      // branch-free: every row computes its derivatives; rows outside an
      // update domain keep their value, rows outside a strip their plain
      // derivative (selects)
      float Dx = st4(b3[kk], b2[kk], b1[kk], b0[kk]) * a.dxI;
      float Dz = st4(z3[kk - 3], z3[kk - 2], z3[kk - 1], z3[kk]) * a.dzI;
      float Dx2 = st4(z3[kk - 3], b2[2 * R8 + kk - 3], b1[2 * R8 + kk - 3], b0[2 * R8 + kk - 3]) * a.dxI;
      float Dz2 = st4(zz[kk - 3], zz[kk - 2], zz[kk - 1], zz[kk]) * a.dzI;
      if constexpr (XPSI) {
        const int j0 = pml_slot(cc - 3, nx - 3, npml, xlo, xhi), j1 = pml_slot(cc - 3, nx - 6, npml, xlo, xhi);
        if (j0 >= 0) Dx = cpml_xs(Dx, 0, j0, PXs(0, s)[q], vxb, psB(0) + XS(j0, q), ownx);
        if (j1 >= 0) Dx2 = cpml_xs(Dx2, 1, j1, PXs(1, s)[q], vzb, psB(1) + XS(j1, q), ownz);
      }
      if (wzv) {
        Dz = cpml_zs(Dz, cq3, PZs(1, s)[jq3c], jq3v >= 0, psB(3) + ZS(cc, jq3c), ownx);
        Dz2 = cpml_zs(Dz2, cq2, PZs(0, s)[jq2c], jq2v >= 0, psB(2) + ZS(cc, jq2c), ownz);
      }
      float vx = vxb ? v0[k] - v0[2 * R4 + k] * (Dx + Dz) : v0[k];
      float vz = vzb ? v0[R4 + k] - v0[3 * R4 + k] * (Dx2 + Dz2) : v0[R4 + k];
      if (gany) {
        const float g = __shfl_sync(0xffffffffu, vz, glane);
        if (gsrc) vz = gok ? -g : -vz_any(gsrc, cc);
      }
      // add_velocity_source! (after the mirrors took their values)
      if (ib0 < ie0) inject(a.cells, a.amount, ib0, ie0, q, vx);
      if (ib1 < ie1) inject(a.cells, a.amount, ib1, ie1, q, vz);
      if (vact) {
        svx[s * R4 + k] = vx;
        svz[s * R4 + k] = vz;
      }
      const int64_t o = so + S(q, cc);
      if (ownx) a.vxB[o] = vx;
      if (ownz) a.vzB[o] = vz;
    };
    // stresses of column c from velocity slots s0..s3 = columns c..c+3;
    // halo lanes recompute the last row and store nothing
    // (cells of the column's stress sources in [bs, es))
    auto str_band = [&](int c, int s0, int s1, int s2, int s3, int bs, int es) {
      const int k = t < TZ ? t : TZ - 1, rk = z0 + k;
      const float *u0 = svx + s0 * R4, *u1 = svx + s1 * R4, *u2 = svx + s2 * R4, *u3 = svx + s3 * R4;
      const float *w0 = svz + s0 * R4, *w1 = svz + s1 * R4, *w2 = svz + s2 * R4, *w3 = svz + s3 * R4;
      const float *bc = ring + s0 * SL, *cf = bc + 3 * R8 + 4 * R4;
      float dvxdx = st4(u0[k], u1[k], u2[k], u3[k]) * a.dxI;
      float dvzdz = st4(w0[k], w0[k + 1], w0[k + 2], w0[k + 3]) * a.dzI;
      float dvxdz = st4(u3[k], u3[k + 1], u3[k + 2], u3[k + 3]) * a.dzI;
      float dvzdx = st4(w0[k + 3], w1[k + 3], w2[k + 3], w3[k + 3]) * a.dxI;
      if constexpr (XPSI) {
        const int j4 = pml_slot(c, nx, npml, xlo, xhi), j7 = pml_slot(c, nx - 3, npml, xlo, xhi);
        if (j4 >= 0) dvxdx = cpml_xs(dvxdx, 4, j4, PXs(2, s0)[rk], srow, psB(4) + XS(j4, rk), true);
        if (j7 >= 0) dvzdx = cpml_xs(dvzdx, 7, j7, PXs(3, s0)[rk], srow && xzrow, psB(7) + XS(j7, rk), true);
      }
      if (wzs) {
        dvzdz = cpml_zs(dvzdz, cr5, PZs(2, s0)[jr5c], jr5v >= 0, psB(5) + ZS(c, jr5c), true);
        dvxdz = cpml_zs(dvxdz, cr6, PZs(3, s0)[jr6c], jr6v >= 0, psB(6) + ZS(c, jr6c), true);
      }
      const float M = cf[k], Lm = cf[TZ + k], mu = cf[2 * TZ + k];
      float txx = bc[k + 4] - (M * dvxdx) - (Lm * (dvzdz));
      float tzz = bc[R8 + k + 4] - (M * dvzdz) - (Lm * (dvxdx));
      float txz = bc[2 * R8 + k + 4] - mu * (dvxdz + dvzdx);
      if (fsblk) {
        // free_surface_mirror!(tauzz), free_surface!(tauxz): tzz[1] = -tzz[2]
        const float t2 = __shfl_down_sync(0xffffffffu, tzz, 1);
        if (fsrow) {
          tzz = -t2;
          txz = 0.f;
        }
      }
      // add_stress_source!: txx += pv dtM; tzz += pv dtM
      if (bs < es) {
        inject(a.cells, a.amount, bs, es, r, txx);
        inject(a.cells, a.amount, bs, es, r, tzz);
      }
      if (srow) {
        const int64_t o = so + S(r, c);
        a.txxB[o] = txx;
        a.tzzB[o] = tzz;
        if (xzrow) a.txzB[o] = txz;
      }
    };
    if constexpr (MODE == 1 || MODE == 2) {
      // iteration it handles column c = xbase + it: slot(c + m) = (it + m) % RING
      const int ncol = x1 - xbase;
      // a rolled loop: the band code unrolled by the ring length overflows
      // the instruction cache
      for (int it = 0; it < ncol; it++) {
        const int c = xbase + it, cc = c + 3;
        int ib0, ie0, ib1, ie1, bs = 0, es = 0;
        cvx.range(a.cells, cc, ib0, ie0);
        cvz.range(a.cells, cc, ib1, ie1);
        if (c >= x0) cst.range(a.cells, c, bs, es);
        if (!mbar_wait(&bar[(it + 3) % RING], ((it + 3) / RING) & 1)) s_err = 1;
        vel_band(cc, it % RING, (it + 1) % RING, (it + 2) % RING, (it + 3) % RING, ib0, ie0, ib1, ie1);
        __syncthreads();
        if constexpr (MODE == 1) {
          if (issuer && it >= 1 && c + RING - 1 <= xlast) issue_fast((it + RING - 1) % RING);
        } else {
          if (issuer) issue(c + RING - 1);
        }
        if (c >= x0) str_band(c, it % RING, (it + 1) % RING, (it + 2) % RING, (it + 3) % RING, bs, es);
      }
    } else {
      // velocities of column cc: update_v! with CPML, mirrors, sources
      auto vel_edge = [&](int cc, int ib0, int ie0, int ib1, int ie1) {
        if (!vact) return;
        const int k = kq, kk = kq + 4, s = slot(cc);
        const bool vxc = cc >= 4 && cc <= nx, vzc = cc >= 4 && cc <= nx - 3;
        const int j0 = pml_slot(cc - 3, nx - 3, npml, xlo, xhi), j1 = pml_slot(cc - 3, nx - 6, npml, xlo, xhi);
        const bool ownc = cc >= x0 && (cc < x1 || lastx);
        const bool ownx = ownc && ownr && q <= nz, ownz = ownc && ownr && cc <= nx && q <= nz + 3;
        const float *b3 = ring + slot(cc - 3) * SL, *b2 = ring + slot(cc - 2) * SL,
                    *b1 = ring + slot(cc - 1) * SL, *bq = ring + s * SL;
        const float *v0 = bq + 3 * R8, *z3 = b3 + 2 * R8;
        float vx;
        if (rxhi && cc >= nx + 2) {
          vx = cc == nx + 3 ? -vpre : -svx[slot(cc - 1) * R4 + k];  // vx[nx+3] = -vx[nx], vx[nx+2] = -vx[nx+1]
        } else {
          vx = v0[k];
          if (vxr && vxc) {
            float Dx = st4(b3[kk], b2[kk], b1[kk], bq[kk]) * a.dxI;
            if (j0 >= 0) Dx = cpml_p(Dx, 0, j0, PX(0, cc)[q], psB(0) + XS(j0, q), ownx);
            float Dz = st4(z3[kk - 3], z3[kk - 2], z3[kk - 1], z3[kk]) * a.dzI;
            if (jq3 >= 0) Dz = cpml_z(Dz, cq3, PZ(1, cc)[jq3], psB(3) + ZS(cc, jq3), ownx);
            vx = vx - v0[2 * R4 + k] * (Dx + Dz);
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
        if (!a.vonly) inject(a.cells, a.amount, ib0, ie0, q, vx);
        svx[s * R4 + k] = vx;
        if (ownx) a.vxB[so + S(q, cc)] = vx;
        float vz;
        if (gsrc) {
          vz = -vz_any(gsrc, cc);
        } else {
          vz = v0[R4 + k];
          if (vzr && vzc) {
            float Dx = st4(z3[kk - 3], b2[2 * R8 + kk - 3], b1[2 * R8 + kk - 3], bq[2 * R8 + kk - 3]) * a.dxI;
            if (j1 >= 0) Dx = cpml_p(Dx, 1, j1, PX(1, cc)[q], psB(1) + XS(j1, q), ownz);
            const float *zz = bq + R8;
            float Dz = st4(zz[kk - 3], zz[kk - 2], zz[kk - 1], zz[kk]) * a.dzI;
            if (jq2 >= 0) Dz = cpml_z(Dz, cq2, PZ(0, cc)[jq2], psB(2) + ZS(cc, jq2), ownz);
            vz = vz - v0[3 * R4 + k] * (Dx + Dz);
          }
        }
        if (!a.vonly) inject(a.cells, a.amount, ib1, ie1, q, vz);
        svz[s * R4 + k] = vz;
        if (ownz) a.vzB[so + S(q, cc)] = vz;
      };
      // stresses of column c: compute_stressii!/ij!, free surface, sources
      auto str_edge = [&](int c, int bs, int es) {
        if (!srow) return;
        const int k = t;
        const int j4 = pml_slot(c, nx, npml, xlo, xhi), j7 = pml_slot(c, nx - 3, npml, xlo, xhi);
        const float *u0 = svx + slot(c) * R4, *u1 = svx + slot(c + 1) * R4, *u2 = svx + slot(c + 2) * R4,
                    *u3 = svx + slot(c + 3) * R4;
        const float *w0 = svz + slot(c) * R4, *w1 = svz + slot(c + 1) * R4, *w2 = svz + slot(c + 2) * R4,
                    *w3 = svz + slot(c + 3) * R4;
        const float *bc = ring + slot(c) * SL, *cf = bc + 3 * R8 + 4 * R4;
        const int64_t o = so + S(r, c);
        const bool hasxz = xzrow && c <= nx - 3;
        float txx, tzz, txz = 0.f;
        if (a.vonly) {
          txx = bc[k + 4];
          tzz = bc[R8 + k + 4];
          txz = bc[2 * R8 + k + 4];
        } else {
          float dvxdx = st4(u0[k], u1[k], u2[k], u3[k]) * a.dxI;
          if (j4 >= 0) dvxdx = cpml_p(dvxdx, 4, j4, PX(2, c)[r], psB(4) + XS(j4, r), true);
          float dvzdz = st4(w0[k], w0[k + 1], w0[k + 2], w0[k + 3]) * a.dzI;
          if (jr5 >= 0) dvzdz = cpml_z(dvzdz, cr5, PZ(2, c)[jr5], psB(5) + ZS(c, jr5), true);
          const float M = cf[k], Lm = cf[TZ + k];
          txx = bc[k + 4] - (M * dvxdx) - (Lm * (dvzdz));
          tzz = bc[R8 + k + 4] - (M * dvzdz) - (Lm * (dvxdx));
          if (hasxz) {
            float dvxdz = st4(u3[k], u3[k + 1], u3[k + 2], u3[k + 3]) * a.dzI;
            if (jr6 >= 0) dvxdz = cpml_z(dvxdz, cr6, PZ(3, c)[jr6], psB(6) + ZS(c, jr6), true);
            float dvzdx = st4(w0[k + 3], w1[k + 3], w2[k + 3], w3[k + 3]) * a.dxI;
            if (j7 >= 0) dvzdx = cpml_p(dvzdx, 7, j7, PX(3, c)[r], psB(7) + XS(j7, r), true);
            txz = bc[2 * R8 + k + 4] - cf[2 * TZ + k] * (dvxdz + dvzdx);
          }
          if (fsrow) {
            // free_surface_mirror!(tauzz), free_surface!(tauxz): tzz[1] = -tzz[2]
            tzz = -tzz_row2(c);
            txz = 0.f;
          }
          // add_stress_source!: txx += pv dtM; tzz += pv dtM
          inject(a.cells, a.amount, bs, es, r, txx);
          inject(a.cells, a.amount, bs, es, r, tzz);
        }
        a.txxB[o] = txx;
        a.tzzB[o] = tzz;
        if (hasxz) a.txzB[o] = txz;
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
    // a wait gave up: let the copies still in flight land before the block's
    // shared memory is released, then report
    for (int cc = max(xbase, xlast - (RING - 1)); cc <= xlast; cc++) {
      const int j = cc - xbase;
      mbar_wait(&bar[j % RING], (j / RING) & 1);
    }
    atomicExch(a.err, 1);
  }
}

template <int MODE>
__global__ void __launch_bounds__(E2_THREADS, MODE == 0 ? 6 : MODE == 1 ? 6 : MODE == 2 ? 4 : 3) k_e2(const E2Args a) {
  e2_body<MODE>(a, a.tiles[blockIdx.x]);
}

// One step of several plans in one launch (a batch, gpi_batch.cu): the
// tiles of every plan of one class, each tagged with its plan's slot in the
// high half of .w; the block copies its plan's arguments for this class and
// buffer parity (args[(slot * 4 + MODE) * 2 + par]) to shared memory.
template <int MODE>
__global__ void __launch_bounds__(E2_THREADS, MODE == 0 ? 6 : MODE == 1 ? 6 : MODE == 2 ? 4 : 3)
    k_e2_batch(const E2Args *__restrict__ args, const int4 *__restrict__ tiles, int par) {
  __shared__ __align__(16) E2Args sa;
  const int4 tile = tiles[blockIdx.x];
  const int slot = tile.w >> 16;
  const int *src = reinterpret_cast<const int *>(args + ((int64_t)slot * 4 + MODE) * 2 + par);
  int *dst = reinterpret_cast<int *>(&sa);
  for (int i = threadIdx.x; i < (int)(sizeof(E2Args) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  e2_body<MODE>(sa, tile);
}

// the arguments of one time step (`flip` swaps the buffers)
static void e2_fill(Plan *p, int vonly, int flip, E2Args &a) {
  a.nz = p->d.nz;
  a.nx = p->d.nx;
  a.NZP = p->NZP;
  a.fs = p->fstride;
  a.npml = p->d.npml;
  a.faces = p->d.pml_faces;
  a.rigid = p->d.rigid_faces;
  a.free = p->d.free_faces;
  a.dxI = (float)(1.0 / (p->d.dx * 24.0));
  a.dzI = (float)(1.0 / (p->d.dz * 24.0));
  a.nzb = p->nzb;
  const int A = p->cur[0] ^ flip, B = A ^ 1;
  a.txxA = p->state[A][0][GPI_TAUXX];
  a.tzzA = p->state[A][0][GPI_TAUZZ];
  a.txzA = p->state[A][0][GPI_TAUXZ];
  a.vxA = p->state[A][0][GPI_VX];
  a.vzA = p->state[A][0][GPI_VZ];
  a.txxB = p->state[B][0][GPI_TAUXX];
  a.tzzB = p->state[B][0][GPI_TAUZZ];
  a.txzB = p->state[B][0][GPI_TAUXZ];
  a.vxB = p->state[B][0][GPI_VX];
  a.vzB = p->state[B][0][GPI_VZ];
  for (int q = 0; q < 8; q++) {
    a.psA[q] = p->psi[A][0][q];
    a.psB[q] = p->psi[B][0][q];
    a.pss[q] = p->psi_stride[q];
  }
  a.cx = p->coef[0];
  a.cz = p->coef[1];
  a.mu = p->coef[2];
  a.dtM = p->coef[3];
  a.dtl = p->coef[4];
  a.pml = p->pml;
  a.cells = p->d_cells;
  a.gptr = p->d_group_ptr;
  a.amount = p->d_amount;
  a.vonly = vonly;
  a.err = p->d_err;
  a.tiles = p->d_tiles;
  a.zsw = p->zsw;
  a.pzw = p->pzw;
  a.psf = 0;
}

// per tile class: CPML floats per ring slot and shared memory per block
static void e2_sizes(const Plan *p, int psf[4], size_t smem[4]) {
  const bool zf = p->d.pml_faces & (GPI_ZMIN | GPI_ZMAX);
  psf[0] = 0;
  psf[1] = zf ? 4 * p->pzw : 0;
  psf[2] = psf[3] = e2_psi_floats(*p);
  for (int m = 0; m < 4; m++) smem[m] = m == 0 ? E2_SMEM : e2_smem_general(psf[m], e2_ring(m));
}

int step_elastic2d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  (void)ipw_mask;
  (void)it;
  (void)mode;
  E2Args a;
  e2_fill(p, vonly, 0, a);
  // shared memory per block: the ring with the CPML memory each mode stages
  int psf[4];
  size_t smem[4];
  e2_sizes(p, psf, smem);
  void (*const fn[4])(E2Args) = {k_e2<0>, k_e2<1>, k_e2<2>, k_e2<3>};
  for (int m = 0; m < 4; m++)
    if (int rc = ensure_smem_attr(p, (const void *)fn[m], 4 + m, smem[m])) return rc;
  auto launch = [&](int m, int first, int n, cudaStream_t st) {
    if (n <= 0) return;
    E2Args g = a;
    g.tiles = p->d_tiles + first;
    g.psf = psf[m];
    fn[m]<<<n, E2_THREADS, smem[m], st>>>(g);
    p->launches++;
  };
  const int *n = p->n_tiles;
  const int ntot = n[0] + n[1] + n[2] + n[3];
  if (vonly) {
    // the velocity-only half step runs every tile on the general code
    launch(3, 0, ntot, p->stream);
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
  p->cur[0] ^= 1;
  return GPI_OK;
}

// --- batches of plans (gpi_batch.cu) ---
size_t e2_args_bytes() { return sizeof(E2Args); }

// a forward plan's arguments per tile class and buffer parity ([class][parity],
// parity 1 with the buffers swapped) and its shared memory per class
void e2_batch_args(Plan *p, void *out, size_t smem[4]) {
  int psf[4];
  e2_sizes(p, psf, smem);
  E2Args *o = static_cast<E2Args *>(out);
  for (int m = 0; m < 4; m++)
    for (int par = 0; par < 2; par++) {
      E2Args &a = o[m * 2 + par];
      e2_fill(p, 0, par, a);
      a.tiles = nullptr;
      a.psf = psf[m];
    }
}

// one launch of tile class m over n tagged tiles of the batch's plans
int e2_batch_launch(Plan *p, int m, const void *args, const int4 *tiles, int n, int par, size_t smem, cudaStream_t st) {
  void (*const fn[4])(const E2Args *, const int4 *, int) = {k_e2_batch<0>, k_e2_batch<1>, k_e2_batch<2>,
                                                             k_e2_batch<3>};
  if (int rc = ensure_smem_attr(p, (const void *)fn[m], 20 + m, smem)) return rc;
  if (n <= 0) return GPI_OK;  // (n = 0: only the kernel's shared-memory attribute)
  fn[m]<<<n, E2_THREADS, smem, st>>>(static_cast<const E2Args *>(args), tiles, par);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

}  // namespace gpi
