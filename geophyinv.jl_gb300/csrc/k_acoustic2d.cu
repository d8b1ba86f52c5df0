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
// Work decomposition: a block owns TZ rows x L columns of p of one shot and
// sweeps its columns left to right.  Pressure columns live in an 8-column
// shared-memory ring (rows z0-3 .. z0+TZ+2), the four vx columns the
// x-derivative needs live in registers, the TZ+3 vz values of the current
// column in shared memory.  The 3 vx columns right of the tile and the 3 vz
// rows below it are recomputed from the input buffer instead of exchanged,
// so the state is ping-ponged between two buffers and a step is one pass
// over HBM: read p, vx, vz, cx, cz, dtK, write p, vx, vz (36 B per cell).
#include <climits>

#include "gpi_internal.cuh"

namespace gpi {

struct A2Args {
  int nz, nx, NZP;
  int64_t fs;
  int npml, faces, rigid;
  float dxI, dzI, dtI;
  int L, nzb, nxb, nshots;
  // wavefield 1 (and 2 in adjoint mode): read buffer A, write buffer B
  const float *pA[2], *vxA[2], *vzA[2];
  float *pB[2], *vxB[2], *vzB[2];
  const float *psA[2][4];
  float *psB[2][4];
  int64_t pss[4];
  const float *cx, *cz, *dtK;
  const float *pml;  // [4][3][2*npml]
  const InjCell *cells;
  const int32_t *gptr;
  const float *amount;
  int vonly;
  // adjoint extras
  const float *bstore;  // this step's strips (shot 0), x strips then z strips
  int64_t bsstride;
  int npx, npz, nb;
  float *gK, *gR;
  float *bufx, *bufz;   // gradient scratch (vx/vz "velocity_buffer" of wavefield 1)
};

__device__ __forceinline__ float st4(float a0, float a1, float a2, float a3) {
  return a2 * 27.0f - a1 * 27.0f + a0 - a3;
}

// CPML strip slot of derivative index i (1-based) on an axis of length nd
__device__ __forceinline__ int pml_slot(int i, int nd, int npml, bool lo, bool hi) {
  if (lo && i <= npml) return i - 1;
  if (hi && i > nd - npml) return npml + i - (nd - npml) - 1;
  return -1;
}

// psi = b psi + a d ; d = d kI + psi   (memory{x,z}!, src/fdtd/cpml.jl:175-182)
__device__ __forceinline__ float cpml(float D, const float *pm, int npml, int j, const float *psA, float *psB,
                                      int64_t po, bool own) {
  const float psi = pm[2 * npml + j] * psA[po] + pm[j] * D;
  if (own) psB[po] = psi;
  return D * pm[4 * npml + j] + psi;
}

template <int TZ>
__global__ void __launch_bounds__(TZ) k_a2_forward(const A2Args a) {
  __shared__ float sp[8][TZ + 6];
  __shared__ float svz[2][TZ + 4];
  __shared__ int s_cur[3], s_end[3];
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
  const float *__restrict__ pA = a.pA[0] + so;
  const float *__restrict__ vxA = a.vxA[0] + so;
  const float *__restrict__ vzA = a.vzA[0] + so;
  float *__restrict__ pB = a.pB[0] + so;
  float *__restrict__ vxB = a.vxB[0] + so;
  float *__restrict__ vzB = a.vzB[0] + so;
  const bool xlo = a.faces & GPI_XMIN, xhi = a.faces & GPI_XMAX, zlo = a.faces & GPI_ZMIN, zhi = a.faces & GPI_ZMAX;
  const bool rxlo = a.rigid & GPI_XMIN, rxhi = a.rigid & GPI_XMAX, rzlo = a.rigid & GPI_ZMIN, rzhi = a.rigid & GPI_ZMAX;
  const float *psA[4];
  float *psB[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    psA[q] = a.psA[0][q] ? a.psA[0][q] + shot * a.pss[q] : nullptr;
    psB[q] = a.psB[0][q] ? a.psB[0][q] + shot * a.pss[q] : nullptr;
  }
  const float *pm0 = a.pml, *pm1 = a.pml + 6 * npml, *pm2 = a.pml + 12 * npml, *pm3 = a.pml + 18 * npml;
  const int r = z0 + t;
  auto S = [&](int rr, int cc) -> int64_t { return (int64_t)(cc + XOFF - 1) * NZP + (rr + ZOFF - 1); };

  // injection cursors (cells sorted by column) for vx, vz and p
  if (t < 3) {
    const int kind = t == 0 ? 0 : t == 1 ? 2 : 3;
    const int g = shot * NKIND + kind;
    int lo = a.gptr[g], hi = a.gptr[g + 1];
    const int end = hi;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (a.cells[mid].col < x0)
        lo = mid + 1;
      else
        hi = mid;
    }
    s_cur[t] = lo;
    s_end[t] = end;
  }

  auto load_p = [&](int cc) {
    float *dst = sp[cc & 7];
    for (int k = t; k < TZ + 6; k += TZ) dst[k] = pA[S(z0 - 3 + k, cc)];
  };
  // vx before the source (update_v! incl. CPML of dpdx)
  auto vx_upd = [&](int cc, bool own) -> float {
    const int64_t o = S(r, cc);
    float v = vxA[o];
    if (r >= 4 && r <= nz - 3 && cc >= 4 && cc <= nx) {
      float D = st4(sp[(cc - 3) & 7][t + 3], sp[(cc - 2) & 7][t + 3], sp[(cc - 1) & 7][t + 3], sp[cc & 7][t + 3]) * a.dxI;
      const int j = pml_slot(cc - 3, nx - 3, npml, xlo, xhi);
      if (j >= 0) D = cpml(D, pm0, npml, j, psA[0], psB[0], (int64_t)j * NZP + (r + ZOFF - 1), own);
      v = v + a.cx[o] * D;
    }
    return v;
  };
  auto vz_upd = [&](int q, int cc, bool own) -> float {
    const int64_t o = S(q, cc);
    float v = vzA[o];
    if (q >= 4 && q <= nz && cc >= 4 && cc <= nx - 3) {
      const float *col = sp[cc & 7];
      const int k = q - z0;
      float D = st4(col[k], col[k + 1], col[k + 2], col[k + 3]) * a.dzI;
      const int j = pml_slot(q - 3, nz - 3, npml, zlo, zhi);
      if (j >= 0) D = cpml(D, pm1, npml, j, psA[1], psB[1], (int64_t)(cc + XOFF - 1) * 2 * npml + j, own);
      v = v + a.cz[o] * D;
    }
    return v;
  };
  auto inj = [&](int b, int e, int row, float &v) {
    if (a.vonly) return;  // the extra half step after the loop adds no sources
    for (int k = b; k < e; k++)
      if (a.cells[k].row == row) v = v + a.amount[k];
  };

  __syncthreads();
  int cur0 = s_cur[0], end0 = s_end[0], cur1 = s_cur[1], end1 = s_end[1], cur2 = s_cur[2], end2 = s_end[2];
  int ncol0 = cur0 < end0 ? a.cells[cur0].col : INT_MAX;
  int ncol1 = cur1 < end1 ? a.cells[cur1].col : INT_MAX;
  int ncol2 = cur2 < end2 ? a.cells[cur2].col : INT_MAX;
  auto range = [&](int &cur, int end, int &ncol, int col, int &b, int &e) {
    b = cur;
    if (ncol == col) {
      while (cur < end && a.cells[cur].col == col) cur++;
      ncol = cur < end ? a.cells[cur].col : INT_MAX;
    }
    e = cur;
  };

  const bool rown = r <= nz;  // vx and p rows
  float vpre_nx = 0.f;        // vx[r, nx] before its source (xmax mirror)
  float u0 = 0.f, u1 = 0.f, u2 = 0.f, u3 = 0.f;
  // one vx column: update, mirrors, source, store
  auto vx_col = [&](int cc, float um3, float um2) -> float {
    // um3 / um2: vx at cc-2 / cc-1 (only used by the xmax mirror)
    const bool own = rown && cc >= x0 && (cc < x1 || lastx);
    float v;
    if (rxhi && cc >= nx + 2) {
      v = cc == nx + 3 ? -vpre_nx : -um2;  // vx[nx+3] = -vx[nx], vx[nx+2] = -vx[nx+1]
    } else {
      v = vx_upd(cc, own);
      if (cc == nx) vpre_nx = v;
    }
    int b, e;
    range(cur0, end0, ncol0, cc, b, e);
    inj(b, e, r, v);
    if (own) vxB[S(r, cc)] = v;
    return v;
  };

  // ---- prologue: p columns x0-3 .. x0+2, vx columns x0 .. x0+2 ----
  for (int cc = x0 - 3; cc <= x0 + 2; cc++) load_p(cc);
  __syncthreads();
  u0 = vx_col(x0, 0.f, 0.f);
  u1 = vx_col(x0 + 1, 0.f, u0);
  u2 = vx_col(x0 + 2, u0, u1);

  for (int c = x0; c < x1; c++) {
    load_p(c + 3);
    __syncthreads();
    // vx column c+3
    u3 = vx_col(c + 3, u1, u2);
    if (rxlo && c + 3 == 4) {
      // dirichletxmin!: vx[1] = -vx[4], vx[2] = -vx[3] (vx[4] before its source)
      const float pre = vx_upd(4, false);
      u0 = -pre;
      u1 = -u2;
      if (rown && x0 == 1) {
        vxB[S(r, 1)] = u0;
        vxB[S(r, 2)] = u1;
      }
    }
    // vz column c, rows z0 .. z0+TZ+2
    {
      int b, e;
      range(cur1, end1, ncol1, c, b, e);
      for (int k = t; k < TZ + 3; k += TZ) {
        const int q = z0 + k;
        const bool own = (k < TZ || lastz) && q <= nz + 3 && c < x1;
        float v;
        if (rzlo && q <= 2)
          v = -vz_upd(5 - q, c, false);  // dirichletzmin!: vz[1] = -vz[4], vz[2] = -vz[3]
        else if (rzhi && q >= nz + 2)
          v = -vz_upd(2 * nz + 3 - q, c, false);  // dirichletzmax!
        else
          v = vz_upd(q, c, own);
        inj(b, e, q, v);
        svz[c & 1][k] = v;
        if (own) vzB[S(q, c)] = v;
      }
    }
    __syncthreads();
    // p at (r, c)
    {
      int b, e;
      range(cur2, end2, ncol2, c, b, e);
      if (rown) {
        const int64_t o = S(r, c);
        const float pold = sp[c & 7][t + 3];
        float pn;
        if (a.vonly) {
          pn = pold;
        } else {
          float Dx = st4(u0, u1, u2, u3) * a.dxI;
          int j = pml_slot(c, nx, npml, xlo, xhi);
          if (j >= 0) Dx = cpml(Dx, pm2, npml, j, psA[2], psB[2], (int64_t)j * NZP + (r + ZOFF - 1), true);
          const float *vz = svz[c & 1];
          float Dz = st4(vz[t], vz[t + 1], vz[t + 2], vz[t + 3]) * a.dzI;
          j = pml_slot(r, nz, npml, zlo, zhi);
          if (j >= 0) Dz = cpml(Dz, pm3, npml, j, psA[3], psB[3], (int64_t)(c + XOFF - 1) * 2 * npml + j, true);
          pn = pold + (Dx + Dz) * a.dtK[o];
          inj(b, e, r, pn);
        }
        pB[o] = pn;
      }
    }
    u0 = u1;
    u1 = u2;
    u2 = u3;
  }
}

int step_adjoint_acoustic2d(Plan *p, int it);

static void fill_args(Plan *p, A2Args &a) {
  a.nz = p->d.nz;
  a.nx = p->d.nx;
  a.NZP = p->NZP;
  a.fs = p->fstride;
  a.npml = p->d.npml;
  a.faces = p->d.pml_faces;
  a.rigid = p->d.rigid_faces;
  const double den = 24.0;
  a.dxI = (float)(1.0 / (p->d.dx * den));
  a.dzI = (float)(1.0 / (p->d.dz * den));
  a.dtI = (float)(1.0 / p->d.dt);
  a.L = p->L;
  a.nzb = p->nzb;
  a.nxb = p->nxb;
  a.nshots = p->d.nshots;
  for (int w = 0; w < 2; w++) {
    const int A = p->cur[w], B = p->cur[w] ^ 1;
    const int ww = w < p->d.npw ? w : 0;
    a.pA[w] = p->state[A][ww][GPI_P];
    a.vxA[w] = p->state[A][ww][GPI_VX];
    a.vzA[w] = p->state[A][ww][GPI_VZ];
    a.pB[w] = p->state[B][ww][GPI_P];
    a.vxB[w] = p->state[B][ww][GPI_VX];
    a.vzB[w] = p->state[B][ww][GPI_VZ];
    for (int q = 0; q < 4; q++) {
      a.psA[w][q] = p->psi[A][ww][q];
      a.psB[w][q] = p->psi[B][ww][q];
    }
  }
  for (int q = 0; q < 4; q++) a.pss[q] = p->psi_stride[q];
  a.cx = p->coef[0];
  a.cz = p->coef[1];
  a.dtK = p->coef[2];
  a.pml = p->pml;
  a.cells = p->d_cells;
  a.gptr = p->d_group_ptr;
  a.amount = p->d_amount;
  a.vonly = 0;
  a.bstore = nullptr;
  a.bsstride = 0;
  a.npx = a.npz = a.nb = 0;
  a.gK = a.gR = nullptr;
  a.bufx = a.bufz = nullptr;
}

int step_acoustic2d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  if (mode == GPI_ADJOINT && !vonly) return step_adjoint_acoustic2d(p, it);
  (void)ipw_mask;
  A2Args a;
  fill_args(p, a);
  a.vonly = vonly;
  const int blocks = p->nzb * p->nxb * p->d.nshots;
  k_a2_forward<128><<<blocks, 128, 0, p->stream>>>(a);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  p->cur[0] ^= 1;
  return GPI_OK;
}

int step_adjoint_acoustic2d(Plan *p, int it) {
  (void)it;
  return fail(p, GPI_E_UNSUPPORTED, "adjoint step not built yet");
}

}  // namespace gpi
