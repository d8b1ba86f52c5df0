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
// A block owns TZ rows x L columns of the normal-stress grid of one shot and
// sweeps its columns.  The three stress fields stream through an 8-column
// shared-memory ring (rows z0-3 .. z0+TZ+2); the velocities of the 4 columns
// the stress update needs sit in a 4-column ring (rows z0 .. z0+TZ+2).  Halo
// velocities are recomputed from the input buffer (ping-pong state), so a
// step is one pass over HBM: read 5 state + 5 coefficient arrays, write 5
// state arrays (60 B per cell).
#include "k_stencil.cuh"

namespace gpi {

struct E2Args {
  int nz, nx, NZP;
  int64_t fs;
  int npml, faces, rigid, free;
  float dxI, dzI;
  int L, nzb, nxb;
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
};

template <int TZ>
__global__ void __launch_bounds__(TZ) k_e2(const E2Args a) {
  constexpr int TR = TZ + 6;  // stress ring rows: z0-3 .. z0+TZ+2
  constexpr int VR = TZ + 3;  // velocity ring rows: z0 .. z0+TZ+2
  __shared__ float sxx[8][TR], szz[8][TR], sxz[8][TR];
  __shared__ float svx[4][VR], svz[4][VR];
  __shared__ int s_rng[3][2];
  const int t = threadIdx.x;
  int bid = blockIdx.x;
  const int zb = bid % a.nzb;
  bid /= a.nzb;
  const int xb = bid % a.nxb;
  const int shot = bid / a.nxb;
  const int z0 = 1 + zb * TZ, x0 = 1 + xb * a.L;
  const int x1 = min(x0 + a.L, a.nx + 1);
  const bool lastx = xb == a.nxb - 1, lastz = zb == a.nzb - 1;
  const int nz = a.nz, nx = a.nx, npml = a.npml, NZP = a.NZP;
  const int64_t so = (int64_t)shot * a.fs;
  const float *__restrict__ txxA = a.txxA + so;
  const float *__restrict__ tzzA = a.tzzA + so;
  const float *__restrict__ txzA = a.txzA + so;
  const float *__restrict__ vxA = a.vxA + so;
  const float *__restrict__ vzA = a.vzA + so;
  float *__restrict__ txxB = a.txxB + so;
  float *__restrict__ tzzB = a.tzzB + so;
  float *__restrict__ txzB = a.txzB + so;
  float *__restrict__ vxB = a.vxB + so;
  float *__restrict__ vzB = a.vzB + so;
  const bool xlo = a.faces & GPI_XMIN, xhi = a.faces & GPI_XMAX, zlo = a.faces & GPI_ZMIN, zhi = a.faces & GPI_ZMAX;
  const bool rxlo = a.rigid & GPI_XMIN, rxhi = a.rigid & GPI_XMAX, rzlo = a.rigid & GPI_ZMIN, rzhi = a.rigid & GPI_ZMAX;
  const bool fsurf = a.free & GPI_ZMIN;
  const float *psA[8];
  float *psB[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    psA[q] = a.psA[q] ? a.psA[q] + shot * a.pss[q] : nullptr;
    psB[q] = a.psB[q] ? a.psB[q] + shot * a.pss[q] : nullptr;
  }
  const int P6 = 6 * npml;  // floats per derivative in a.pml
  auto S = [&](int rr, int cc) -> int64_t { return (int64_t)(cc + XOFF - 1) * NZP + (rr + ZOFF - 1); };
  auto XS = [&](int j, int rr) -> int64_t { return (int64_t)j * NZP + (rr + ZOFF - 1); };        // x strip
  auto ZS = [&](int cc, int j) -> int64_t { return (int64_t)(cc + XOFF - 1) * 2 * npml + j; };   // z strip

  if (t < 3) {
    const int kind = t == 0 ? 0 : t == 1 ? 2 : 3;
    const int g = shot * NKIND + kind;
    s_rng[t][0] = first_col(a.cells, a.gptr[g], a.gptr[g + 1], x0);
    s_rng[t][1] = a.gptr[g + 1];
  }

  auto load_tau = [&](int cc) {
    const int s = cc & 7;
    for (int k = t; k < TR; k += TZ) {
      const int64_t o = S(z0 - 3 + k, cc);
      sxx[s][k] = txxA[o];
      szz[s][k] = tzzA[o];
      sxz[s][k] = txzA[o];
    }
  };
  // vx at (q, cc) before its source (k = q - z0 indexes the rings)
  auto vx_upd = [&](int q, int cc, bool own) -> float {
    const int64_t o = S(q, cc);
    float v = vxA[o];
    if (q >= 4 && q <= nz - 3 && cc >= 4 && cc <= nx) {
      const int k = q - z0 + 3;  // stress-ring row of q
      float Dx = st4(sxx[(cc - 3) & 7][k], sxx[(cc - 2) & 7][k], sxx[(cc - 1) & 7][k], sxx[cc & 7][k]) * a.dxI;
      int j = pml_slot(cc - 3, nx - 3, npml, xlo, xhi);
      if (j >= 0) Dx = cpml(Dx, a.pml + 0 * P6, npml, j, psA[0], psB[0], XS(j, q), own);
      const float *cz = sxz[(cc - 3) & 7];
      float Dz = st4(cz[k - 3], cz[k - 2], cz[k - 1], cz[k]) * a.dzI;
      j = pml_slot(q - 3, nz - 6, npml, zlo, zhi);
      if (j >= 0) Dz = cpml(Dz, a.pml + 3 * P6, npml, j, psA[3], psB[3], ZS(cc, j), own);
      v = v - a.cx[o] * (Dx + Dz);
    }
    return v;
  };
  auto vz_upd = [&](int q, int cc, bool own) -> float {
    const int64_t o = S(q, cc);
    float v = vzA[o];
    if (q >= 4 && q <= nz && cc >= 4 && cc <= nx - 3) {
      const int k = q - z0 + 3;
      float Dx = st4(sxz[(cc - 3) & 7][k - 3], sxz[(cc - 2) & 7][k - 3], sxz[(cc - 1) & 7][k - 3], sxz[cc & 7][k - 3]) *
                 a.dxI;
      int j = pml_slot(cc - 3, nx - 6, npml, xlo, xhi);
      if (j >= 0) Dx = cpml(Dx, a.pml + 1 * P6, npml, j, psA[1], psB[1], XS(j, q), own);
      const float *zz = szz[cc & 7];
      float Dz = st4(zz[k - 3], zz[k - 2], zz[k - 1], zz[k]) * a.dzI;
      j = pml_slot(q - 3, nz - 3, npml, zlo, zhi);
      if (j >= 0) Dz = cpml(Dz, a.pml + 2 * P6, npml, j, psA[2], psB[2], ZS(cc, j), own);
      v = v - a.cz[o] * (Dx + Dz);
    }
    return v;
  };

  __syncthreads();
  InjCursor cvx, cvz, cst;
  cvx.init(a.cells, s_rng[0][0], s_rng[0][1]);
  cvz.init(a.cells, s_rng[1][0], s_rng[1][1]);
  cst.init(a.cells, s_rng[2][0], s_rng[2][1]);

  // pre-source vx at column nx for the rows this thread computes (xmax mirror)
  float vpre[2] = {0.f, 0.f};
  // velocities of column cc for rows z0+k, k = t and t+TZ (< VR): update,
  // mirrors, sources; stored in the rings and (owned) in buffer B
  auto vel_col = [&](int cc) {
    int b0, e0, b1, e1;
    cvx.range(a.cells, cc, b0, e0);
    cvz.range(a.cells, cc, b1, e1);
    const int s = cc & 3;
    const bool ownc = cc >= x0 && (cc < x1 || lastx);
    int i = 0;
    for (int k = t; k < VR; k += TZ, i++) {
      const int q = z0 + k;
      const bool ownr = k < TZ || lastz;
      // vx
      float vx;
      if (rxhi && cc >= nx + 2) {
        vx = cc == nx + 3 ? -vpre[i] : -svx[(cc - 1) & 3][k];  // vx[nx+3] = -vx[nx], vx[nx+2] = -vx[nx+1]
      } else {
        vx = vx_upd(q, cc, ownc && ownr && q <= nz);
        if (cc == nx) vpre[i] = vx;
      }
      if (!a.vonly) inject(a.cells, a.amount, b0, e0, q, vx);
      svx[s][k] = vx;
      if (ownc && ownr && q <= nz) vxB[S(q, cc)] = vx;
      if (rxlo && cc == 4) {
        // dirichletxmin!: vx[1] = -vx[4] (before its source), vx[2] = -vx[3]
        const float pre = vx_upd(q, 4, false);
        svx[1][k] = -pre;
        svx[2][k] = -svx[3][k];
        if (x0 == 1 && ownr && q <= nz) {
          vxB[S(q, 1)] = svx[1][k];
          vxB[S(q, 2)] = svx[2][k];
        }
      }
      // vz
      float vz;
      if (rzlo && q <= 2)
        vz = -vz_upd(5 - q, cc, false);  // dirichletzmin!
      else if (rzhi && q >= nz + 2)
        vz = -vz_upd(2 * nz + 3 - q, cc, false);  // dirichletzmax!
      else
        vz = vz_upd(q, cc, ownc && ownr && cc <= nx);
      if (!a.vonly) inject(a.cells, a.amount, b1, e1, q, vz);
      svz[s][k] = vz;
      if (ownc && ownr && cc <= nx && q <= nz + 3) vzB[S(q, cc)] = vz;
    }
  };

  // stresses at (r, c) from the velocity rings; returns tzz before sources
  const int r = z0 + t;
  auto txx_tzz = [&](int rr, int c, int k, float &txx, float &tzz, bool own) {
    const int64_t o = S(rr, c);
    const float *u0 = svx[c & 3], *u1 = svx[(c + 1) & 3], *u2 = svx[(c + 2) & 3], *u3 = svx[(c + 3) & 3];
    const float *w = svz[c & 3];
    float dvxdx = st4(u0[k], u1[k], u2[k], u3[k]) * a.dxI;
    int j = pml_slot(c, nx, npml, xlo, xhi);
    if (j >= 0) dvxdx = cpml(dvxdx, a.pml + 4 * P6, npml, j, psA[4], psB[4], XS(j, rr), own);
    float dvzdz = st4(w[k], w[k + 1], w[k + 2], w[k + 3]) * a.dzI;
    j = pml_slot(rr, nz, npml, zlo, zhi);
    if (j >= 0) dvzdz = cpml(dvzdz, a.pml + 5 * P6, npml, j, psA[5], psB[5], ZS(c, j), own);
    const float M = a.dtM[o], Lm = a.dtl[o];
    const int kk = k + 3;
    txx = sxx[c & 7][kk] - (M * dvxdx) - (Lm * (dvzdz));
    tzz = szz[c & 7][kk] - (M * dvzdz) - (Lm * (dvxdx));
  };

  // ---- prologue ----
  for (int cc = x0 - 3; cc <= x0 + 2; cc++) load_tau(cc);
  __syncthreads();
  for (int cc = x0; cc <= x0 + 2; cc++) vel_col(cc);

  for (int c = x0; c < x1; c++) {
    load_tau(c + 3);
    __syncthreads();
    vel_col(c + 3);
    __syncthreads();
    int bs, es;
    cst.range(a.cells, c, bs, es);
    if (r <= nz) {
      const int64_t o = S(r, c);
      const int k = t;
      float txx, tzz, txz = 0.f;
      const bool hasxz = r <= nz - 3 && c <= nx - 3;
      if (a.vonly) {
        txx = sxx[c & 7][k + 3];
        tzz = szz[c & 7][k + 3];
        txz = sxz[c & 7][k + 3];
      } else {
        txx_tzz(r, c, k, txx, tzz, true);
        if (hasxz) {
          // compute_stressij!: txz -= mu (dvxdz + dvzdx)
          float dvxdz = st4(svx[(c + 3) & 3][k], svx[(c + 3) & 3][k + 1], svx[(c + 3) & 3][k + 2],
                            svx[(c + 3) & 3][k + 3]) * a.dzI;
          int j = pml_slot(r, nz - 3, npml, zlo, zhi);
          if (j >= 0) dvxdz = cpml(dvxdz, a.pml + 6 * P6, npml, j, psA[6], psB[6], ZS(c, j), true);
          float dvzdx = st4(svz[c & 3][k + 3], svz[(c + 1) & 3][k + 3], svz[(c + 2) & 3][k + 3],
                            svz[(c + 3) & 3][k + 3]) * a.dxI;
          j = pml_slot(c, nx - 3, npml, xlo, xhi);
          if (j >= 0) dvzdx = cpml(dvzdx, a.pml + 7 * P6, npml, j, psA[7], psB[7], XS(j, r), true);
          txz = sxz[c & 7][k + 3] - a.mu[o] * (dvxdz + dvzdx);
        }
        if (fsurf && r == 1) {
          // free_surface_mirror!(tauzz), free_surface!(tauxz): tzz[1] = -tzz[2]
          float t2x, t2z;
          txx_tzz(2, c, 1, t2x, t2z, false);
          tzz = -t2z;
          txz = 0.f;
        }
        // add_stress_source!: txx += pv dtM; tzz += pv dtM
        inject(a.cells, a.amount, bs, es, r, txx);
        inject(a.cells, a.amount, bs, es, r, tzz);
      }
      txxB[o] = txx;
      tzzB[o] = tzz;
      if (hasxz) txzB[o] = txz;
    }
  }
}

int step_elastic2d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  (void)ipw_mask;
  (void)it;
  (void)mode;
  E2Args a;
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
  a.L = p->L;
  a.nzb = p->nzb;
  a.nxb = p->nxb;
  const int A = p->cur[0], B = A ^ 1;
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
  const int blocks = p->nzb * p->nxb * p->d.nshots;
  k_e2<128><<<blocks, 128, 0, p->stream>>>(a);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  p->cur[0] ^= 1;
  return GPI_OK;
}

}  // namespace gpi
