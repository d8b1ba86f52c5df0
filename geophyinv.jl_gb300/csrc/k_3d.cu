// k_3d.cu -- 3-D acoustic and elastic time steps (order 4).
//
// A step is two fused passes over the grid, each updating its fields in place
// with the derivatives computed on the fly (the reference materialises every
// derivative field first, src/fdtd/advance_acou.jl:258-313,
// src/fdtd/advance_elastic.jl:10-230):
//   velocity pass: stress (or p) derivatives + memory*! + compute_v!
//   dirichlet{x,y,z}{min,max}! in the reference's face order, velocity sources
//   stress pass:   velocity derivatives + memory*! + compute_stress*! / compute_p!
//   free surface (elastic), stress sources
// Index arithmetic follows the derivative-field tables of the reference
// (src/fields.jl:92-671, src/fdtd/diff3D.jl:62-134, :303-378): a derivative
// D(iz, iy, ix) of shape kinds (kz, ky, kx) reads its source field from
// (iz, iy, ix) (@d_?a) or from (iz, iy, ix) + h on the other two axes
// (@d_?i), and CPML applies on the first and last npml entries of its own
// axis.  Every field shares the padded storage index map, so a thread owns
// the storage cell (r, y, c) of every field it updates.
#include <algorithm>

#include "k_stencil.cuh"

namespace gpi {

struct G3 {
  int nz, ny, nx, NZP, NYP;
  int64_t fs;
  __device__ __forceinline__ int64_t S(int r, int y, int c) const {
    return ((int64_t)(c + XOFF - 1) * NYP + (y + YOFF - 1)) * NZP + (r + ZOFF - 1);
  }
};

// CPML memory of one derivative field: psi = b psi + a D, D = D kI + psi on
// the strips of its axis (memory{x,y,z}!, src/fdtd/cpml.jl:158-215).
struct Mem3 {
  float *psi[18];
  int64_t pss[18];
  const float *pml;  // [q][a | b | kI][2 npml]
  int npml, w;       // w = 2 npml
  int faces;
};

// psi index of derivative index (iz, iy, ix) with strip slot j on `axis`
__device__ __forceinline__ int64_t psi_index(const G3 &g, const Mem3 &m, int axis, int j, int iz, int iy, int ix) {
  if (axis == 2) return ((int64_t)j * g.NYP + (iy + YOFF - 1)) * g.NZP + (iz + ZOFF - 1);
  if (axis == 1) return ((int64_t)(ix + XOFF - 1) * m.w + j) * g.NZP + (iz + ZOFF - 1);
  return ((int64_t)(ix + XOFF - 1) * g.NYP + (iy + YOFF - 1)) * m.w + j;
}

// D of derivative q at index (iz, iy, ix); i = index along its axis, nd the
// derivative field's extent along that axis
__device__ __forceinline__ float mem3(float D, const G3 &g, const Mem3 &m, int shot, int q, int axis, int i, int nd,
                                     int iz, int iy, int ix) {
  const int lo = axis == 0 ? GPI_ZMIN : axis == 1 ? GPI_YMIN : GPI_XMIN;
  const int hi = axis == 0 ? GPI_ZMAX : axis == 1 ? GPI_YMAX : GPI_XMAX;
  const int j = pml_slot(i, nd, m.npml, m.faces & lo, m.faces & hi);
  if (j < 0) return D;
  const float *cf = m.pml + (int64_t)q * 3 * m.w;
  float *ps = m.psi[q] + shot * m.pss[q] + psi_index(g, m, axis, j, iz, iy, ix);
  const float psi = cf[m.w + j] * *ps + cf[j] * D;
  *ps = psi;
  return D * cf[2 * m.w + j] + psi;
}

struct Step3 {
  G3 g;
  Mem3 m;
  float *f[NFIELD];      // fields, shot 0
  const float *cf[8];    // coefficients (storage layout, shared by shots)
  float dzI, dyI, dxI;
  int shot0, nshots;  // shots [shot0, shot0 + nshots) of this launch
};

// thread -> storage cell (r, y, c) of one shot; extents cover n + h on every axis
struct Cell3 {
  int r, y, c, shot;
  bool ok;
};
__device__ __forceinline__ Cell3 cell3(const G3 &g, int shot0, int nshots, int base = 1) {
  Cell3 e;
  e.r = blockIdx.x * blockDim.x + threadIdx.x + base;
  e.y = blockIdx.y * blockDim.y + threadIdx.y + base;
  const int nc = g.nx + 4 - base;
  e.c = (int)(blockIdx.z % nc) + base;
  e.shot = (int)(blockIdx.z / nc);
  e.ok = e.r <= g.nz + 3 && e.y <= g.ny + 3 && e.shot < nshots;
  e.shot += shot0;
  return e;
}

// ---------------------------------------------------------------------------
// acoustic (DA3: dpdx dpdy dpdz dvxdx dvydy dvzdz)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k3_vel_a(const Step3 a) {
  const G3 &g = a.g;
  const Cell3 e = cell3(g, a.shot0, a.nshots, 4);
  if (!e.ok) return;
  const int r = e.r, y = e.y, c = e.c, nz = g.nz, ny = g.ny, nx = g.nx;
  if (r > nz || y > ny || c > nx) return;
  const int64_t so = e.shot * g.fs, o = so + g.S(r, y, c), oc = o - so;
  const float *p = a.f[GPI_P] + so;
  const int64_t sx = (int64_t)g.NYP * g.NZP, sy = g.NZP;
  // every stencil read first (all in the padded storage for r, y, c >= 4)
  const int64_t bx = g.S(r, y, c - 3), by = g.S(r, y - 3, c), bz = g.S(r - 3, y, c);
  float Dx = st4(p[bx], p[bx + sx], p[bx + 2 * sx], p[bx + 3 * sx]) * a.dxI;  // @d_xi(p)
  float Dy = st4(p[by], p[by + sy], p[by + 2 * sy], p[by + 3 * sy]) * a.dyI;  // @d_yi(p)
  float Dz = st4(p[bz], p[bz + 1], p[bz + 2], p[bz + 3]) * a.dzI;              // @d_zi(p)
  const float cx = a.cf[0][oc], cy = a.cf[1][oc], cz = a.cf[2][oc];
  float *vx = a.f[GPI_VX] + o, *vy = a.f[GPI_VY] + o, *vz = a.f[GPI_VZ] + o;
  const float vx0 = *vx, vy0 = *vy, vz0 = *vz;
  // @inn(vx) += dtinvavxirho * dpdx (nz-2h, ny-2h, nx-h)
  if (r <= nz - 3 && y <= ny - 3) {
    Dx = mem3(Dx, g, a.m, e.shot, 0, 2, c - 3, nx - 3, r - 3, y - 3, c - 3);
    *vx = vx0 + cx * Dx;
  }
  // @inn(vy) += dtinvavyirho * dpdy (nz-2h, ny-h, nx-2h)
  if (r <= nz - 3 && c <= nx - 3) {
    Dy = mem3(Dy, g, a.m, e.shot, 1, 1, y - 3, ny - 3, r - 3, y - 3, c - 3);
    *vy = vy0 + cy * Dy;
  }
  // @inn(vz) += dtinvavzirho * dpdz (nz-h, ny-2h, nx-2h)
  if (y <= ny - 3 && c <= nx - 3) {
    Dz = mem3(Dz, g, a.m, e.shot, 2, 0, r - 3, nz - 3, r - 3, y - 3, c - 3);
    *vz = vz0 + cz * Dz;
  }
}

__global__ void __launch_bounds__(256) k3_str_a(const Step3 a) {
  const G3 &g = a.g;
  const Cell3 e = cell3(g, a.shot0, a.nshots);
  if (!e.ok) return;
  const int r = e.r, y = e.y, c = e.c;
  if (r > g.nz || y > g.ny || c > g.nx) return;
  const int64_t so = e.shot * g.fs, o = so + g.S(r, y, c);
  const int64_t sx = (int64_t)g.NYP * g.NZP, sy = g.NZP;
  const float *vx = a.f[GPI_VX] + o, *vy = a.f[GPI_VY] + o, *vz = a.f[GPI_VZ] + o;
  float Dx = st4(vx[0], vx[sx], vx[2 * sx], vx[3 * sx]) * a.dxI;  // @d_xa(vx)
  Dx = mem3(Dx, g, a.m, e.shot, 3, 2, c, g.nx, r, y, c);
  float Dy = st4(vy[0], vy[sy], vy[2 * sy], vy[3 * sy]) * a.dyI;  // @d_ya(vy)
  Dy = mem3(Dy, g, a.m, e.shot, 4, 1, y, g.ny, r, y, c);
  float Dz = st4(vz[0], vz[1], vz[2], vz[3]) * a.dzI;  // @d_za(vz)
  Dz = mem3(Dz, g, a.m, e.shot, 5, 0, r, g.nz, r, y, c);
  // compute_p!: p += (dvxdx + dvzdz + dvydy) * dtK
  a.f[GPI_P][o] = a.f[GPI_P][o] + (Dx + Dz + Dy) * a.cf[3][o - so];
}

// The acoustic stress pass marching along x: a block owns a 32 x 8 (z, y)
// tile of one shot over a run of columns; vx travels in a register queue
// (c .. c+3), the vy and vz planes of column c in shared memory with their
// +3 halos, and the loads of column c+1 are issued before column c is
// computed.  Same arithmetic as k3_str_a.
constexpr int XM_Z = 32, XM_Y = 8;
__global__ void __launch_bounds__(256) k3_str_a_xm(const Step3 a, int ncx) {
  const G3 &g = a.g;
  __shared__ float svy[2][XM_Y + 3][XM_Z];
  __shared__ float svz[2][XM_Y][XM_Z + 3];
  const int tz = threadIdx.x, ty = threadIdx.y;
  const int z0 = 1 + blockIdx.x * XM_Z, y0 = 1 + blockIdx.y * XM_Y;
  const int xc = (int)(blockIdx.z % ncx), shot = a.shot0 + (int)(blockIdx.z / ncx);
  const int c0 = 1 + (int)((int64_t)g.nx * xc / ncx), c1 = 1 + (int)((int64_t)g.nx * (xc + 1) / ncx);
  const int r = z0 + tz, y = y0 + ty;
  const bool own = r <= g.nz && y <= g.ny;
  const int64_t so = shot * g.fs, sx = (int64_t)g.NYP * g.NZP;
  const float *vx = a.f[GPI_VX] + so, *vy = a.f[GPI_VY] + so, *vz = a.f[GPI_VZ] + so;
  float *p = a.f[GPI_P] + so;
  // rows of this thread (clamped into the padded storage: cells past the
  // grid are never used by an owner)
  const int rr = min(r, g.nz + 3), yy = min(y, g.ny + 3);
  const int64_t o0 = g.S(rr, yy, c0);
  // halo rows: vy at y0+8+ty (ty < 3), vz at z0+32+tz (tz < 3)
  const bool hy = ty < 3, hz = tz < 3;
  const int64_t oy = g.S(rr, min(y0 + XM_Y + ty, g.ny + 3), c0) - o0;
  const int64_t oz = g.S(min(z0 + XM_Z + tz, g.nz + 3), yy, c0) - o0;
  // x queue: vx(c .. c+3)
  float q0 = vx[o0], q1 = vx[o0 + sx], q2 = vx[o0 + 2 * sx], q3;
  float ny_vy = vy[o0], ny_h = hy ? vy[o0 + oy] : 0.f, nz_vz = vz[o0], nz_h = hz ? vz[o0 + oz] : 0.f;
  float nq3 = vx[o0 + 3 * sx];
  for (int c = c0, b = 0; c < c1; c++, b ^= 1) {
    const int64_t o = o0 + (int64_t)(c - c0) * sx;
    q3 = nq3;
    svy[b][ty][tz] = ny_vy;
    if (hy) svy[b][XM_Y + ty][tz] = ny_h;
    svz[b][ty][tz] = nz_vz;
    if (hz) svz[b][ty][XM_Z + tz] = nz_h;
    const float p0 = p[o], k0 = a.cf[3][o - so];
    // the next column's loads, in flight while this one is computed
    if (c + 1 < c1) {
      const int64_t on = o + sx;
      nq3 = vx[on + 3 * sx];
      ny_vy = vy[on];
      if (hy) ny_h = vy[on + oy];
      nz_vz = vz[on];
      if (hz) nz_h = vz[on + oz];
    }
    __syncthreads();
    if (own) {
      float Dx = st4(q0, q1, q2, q3) * a.dxI;  // @d_xa(vx)
      Dx = mem3(Dx, g, a.m, shot, 3, 2, c, g.nx, r, y, c);
      float Dy = st4(svy[b][ty][tz], svy[b][ty + 1][tz], svy[b][ty + 2][tz], svy[b][ty + 3][tz]) * a.dyI;  // @d_ya(vy)
      Dy = mem3(Dy, g, a.m, shot, 4, 1, y, g.ny, r, y, c);
      float Dz = st4(svz[b][ty][tz], svz[b][ty][tz + 1], svz[b][ty][tz + 2], svz[b][ty][tz + 3]) * a.dzI;  // @d_za(vz)
      Dz = mem3(Dz, g, a.m, shot, 5, 0, r, g.nz, r, y, c);
      p[o] = p0 + (Dx + Dz + Dy) * k0;
    }
    q0 = q1;
    q1 = q2;
    q2 = q3;
  }
}

// The acoustic velocity pass marching along x (cells from (4, 4, 4), as
// k3_vel_a): p travels in a register queue (c-3 .. c) and its plane c in
// shared memory with the -3 halos in y and z.  Same arithmetic as k3_vel_a.
__global__ void __launch_bounds__(256) k3_vel_a_xm(const Step3 a, int ncx) {
  const G3 &g = a.g;
  __shared__ float sp[2][XM_Y + 3][XM_Z + 3];
  const int tz = threadIdx.x, ty = threadIdx.y;
  const int nz = g.nz, ny = g.ny, nx = g.nx;
  const int z0 = 4 + blockIdx.x * XM_Z, y0 = 4 + blockIdx.y * XM_Y;
  const int xc = (int)(blockIdx.z % ncx), shot = a.shot0 + (int)(blockIdx.z / ncx);
  const int span = nx - 3;
  const int c0 = 4 + (int)((int64_t)span * xc / ncx), c1 = 4 + (int)((int64_t)span * (xc + 1) / ncx);
  const int r = z0 + tz, y = y0 + ty;
  const bool own = r <= nz && y <= ny;
  const int64_t so = shot * g.fs, sx = (int64_t)g.NYP * g.NZP;
  const float *p = a.f[GPI_P] + so;
  const int rr = min(r, nz + 3), yy = min(y, ny + 3);
  const int64_t o0 = g.S(rr, yy, c0);
  const bool hy = ty < 3, hz = tz < 3;
  const int64_t oy = g.S(rr, y0 - 3 + ty, c0) - o0;  // p(r, y0-3+ty, c)
  const int64_t oz = g.S(z0 - 3 + tz, yy, c0) - o0;  // p(z0-3+tz, y, c)
  float q0 = p[o0 - 3 * sx], q1 = p[o0 - 2 * sx], q2 = p[o0 - sx], q3;
  float n3 = p[o0], nh_y = hy ? p[o0 + oy] : 0.f, nh_z = hz ? p[o0 + oz] : 0.f;
  for (int c = c0, b = 0; c < c1; c++, b ^= 1) {
    const int64_t o = o0 + (int64_t)(c - c0) * sx, oc = o - so;
    q3 = n3;
    sp[b][ty + 3][tz + 3] = q3;
    if (hy) sp[b][ty][tz + 3] = nh_y;
    if (hz) sp[b][ty + 3][tz] = nh_z;
    const float cx = a.cf[0][oc], cy = a.cf[1][oc], cz = a.cf[2][oc];
    float *vx = a.f[GPI_VX] + o, *vy = a.f[GPI_VY] + o, *vz = a.f[GPI_VZ] + o;
    const float vx0 = *vx, vy0 = *vy, vz0 = *vz;
    if (c + 1 < c1) {
      const int64_t on = o + sx;
      n3 = p[on];
      if (hy) nh_y = p[on + oy];
      if (hz) nh_z = p[on + oz];
    }
    __syncthreads();
    if (own) {
      float Dx = st4(q0, q1, q2, q3) * a.dxI;  // @d_xi(p)
      float Dy = st4(sp[b][ty][tz + 3], sp[b][ty + 1][tz + 3], sp[b][ty + 2][tz + 3], sp[b][ty + 3][tz + 3]) * a.dyI;
      float Dz = st4(sp[b][ty + 3][tz], sp[b][ty + 3][tz + 1], sp[b][ty + 3][tz + 2], sp[b][ty + 3][tz + 3]) * a.dzI;
      if (r <= nz - 3 && y <= ny - 3) {
        Dx = mem3(Dx, g, a.m, shot, 0, 2, c - 3, nx - 3, r - 3, y - 3, c - 3);
        *vx = vx0 + cx * Dx;
      }
      if (r <= nz - 3 && c <= nx - 3) {
        Dy = mem3(Dy, g, a.m, shot, 1, 1, y - 3, ny - 3, r - 3, y - 3, c - 3);
        *vy = vy0 + cy * Dy;
      }
      if (y <= ny - 3 && c <= nx - 3) {
        Dz = mem3(Dz, g, a.m, shot, 2, 0, r - 3, nz - 3, r - 3, y - 3, c - 3);
        *vz = vz0 + cz * Dz;
      }
    }
    q0 = q1;
    q1 = q2;
    q2 = q3;
  }
}

// ---------------------------------------------------------------------------
// elastic (DE3, canonical order: dtauxxdx dtauxydx dtauxzdx dtauyydy
// dtauxydy dtauyzdy dtauzzdz dtauyzdz dtauxzdz dvxdx dvydy dvzdz dvxdy dvxdz
// dvydx dvydz dvzdx dvzdy)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k3_vel_e(const Step3 a) {
  const G3 &g = a.g;
  const Cell3 e = cell3(g, a.shot0, a.nshots, 4);
  if (!e.ok) return;
  const int r = e.r, y = e.y, c = e.c, nz = g.nz, ny = g.ny, nx = g.nx;
  if (r > nz || y > ny || c > nx) return;
  const int64_t so = e.shot * g.fs, o = so + g.S(r, y, c), oc = o - so;
  const int64_t sx = (int64_t)g.NYP * g.NZP, sy = g.NZP;
  const float *txx = a.f[GPI_TAUXX] + so, *tyy = a.f[GPI_TAUYY] + so, *tzz = a.f[GPI_TAUZZ] + so;
  const float *txy = a.f[GPI_TAUXY] + so, *txz = a.f[GPI_TAUXZ] + so, *tyz = a.f[GPI_TAUYZ] + so;
  const int iz = r - 3, iy = y - 3, ix = c - 3;  // derivative index of the @inn velocity cell
  // every stencil read first (all in the padded storage for r, y, c >= 4),
  // so that the loads of the three components are in flight together
  const int64_t bx = g.S(r, y, c - 3), bi = g.S(iz, iy, ix), by = g.S(r, iy, c), bz = g.S(iz, y, c);
  float D0 = st4(txx[bx], txx[bx + sx], txx[bx + 2 * sx], txx[bx + 3 * sx]) * a.dxI;  // @d_xi(tauxx)
  float D4 = st4(txy[bi], txy[bi + sy], txy[bi + 2 * sy], txy[bi + 3 * sy]) * a.dyI;  // @d_ya(tauxy)
  float D8 = st4(txz[bi], txz[bi + 1], txz[bi + 2], txz[bi + 3]) * a.dzI;              // @d_za(tauxz)
  float D1 = st4(txy[bi], txy[bi + sx], txy[bi + 2 * sx], txy[bi + 3 * sx]) * a.dxI;  // @d_xa(tauxy)
  float D3 = st4(tyy[by], tyy[by + sy], tyy[by + 2 * sy], tyy[by + 3 * sy]) * a.dyI;  // @d_yi(tauyy)
  float D7 = st4(tyz[bi], tyz[bi + 1], tyz[bi + 2], tyz[bi + 3]) * a.dzI;              // @d_za(tauyz)
  float D2 = st4(txz[bi], txz[bi + sx], txz[bi + 2 * sx], txz[bi + 3 * sx]) * a.dxI;  // @d_xa(tauxz)
  float D5 = st4(tyz[bi], tyz[bi + sy], tyz[bi + 2 * sy], tyz[bi + 3 * sy]) * a.dyI;  // @d_ya(tauyz)
  float D6 = st4(tzz[bz], tzz[bz + 1], tzz[bz + 2], tzz[bz + 3]) * a.dzI;              // @d_zi(tauzz)
  const float cx = a.cf[0][oc], cy = a.cf[1][oc], cz = a.cf[2][oc];
  float *vx = a.f[GPI_VX] + o, *vy = a.f[GPI_VY] + o, *vz = a.f[GPI_VZ] + o;
  const float vx0 = *vx, vy0 = *vy, vz0 = *vz;
  const bool inx = r <= nz - 3 && y <= ny - 3, iny = r <= nz - 3 && c <= nx - 3, inz = y <= ny - 3 && c <= nx - 3;
  // CPML memory only where a derivative index can fall into a strip
  // (strips of extent-(n-6) .. extent-(n-3) derivative fields)
  const int np = a.m.npml;
  if (ix <= np || ix > nx - 6 - np || iy <= np || iy > ny - 6 - np || iz <= np || iz > nz - 6 - np) {
    if (inx) {
      D0 = mem3(D0, g, a.m, e.shot, 0, 2, ix, nx - 3, iz, iy, ix);
      D4 = mem3(D4, g, a.m, e.shot, 4, 1, iy, ny - 6, iz, iy, ix);
      D8 = mem3(D8, g, a.m, e.shot, 8, 0, iz, nz - 6, iz, iy, ix);
    }
    if (iny) {
      D1 = mem3(D1, g, a.m, e.shot, 1, 2, ix, nx - 6, iz, iy, ix);
      D3 = mem3(D3, g, a.m, e.shot, 3, 1, iy, ny - 3, iz, iy, ix);
      D7 = mem3(D7, g, a.m, e.shot, 7, 0, iz, nz - 6, iz, iy, ix);
    }
    if (inz) {
      D2 = mem3(D2, g, a.m, e.shot, 2, 2, ix, nx - 6, iz, iy, ix);
      D5 = mem3(D5, g, a.m, e.shot, 5, 1, iy, ny - 6, iz, iy, ix);
      D6 = mem3(D6, g, a.m, e.shot, 6, 0, iz, nz - 3, iz, iy, ix);
    }
  }
  // vx: @inn(vx) -= dtinvavxirho (dtauxxdx + dtauxydy + dtauxzdz), (nz-2h, ny-2h, nx-h)
  if (inx) *vx = vx0 - cx * (D0 + D4 + D8);
  // vy: @inn(vy) -= dtinvavyirho (dtauxydx + dtauyydy + dtauyzdz), (nz-2h, ny-h, nx-2h)
  if (iny) *vy = vy0 - cy * (D1 + D3 + D7);
  // vz: @inn(vz) -= dtinvavzirho (dtauxzdx + dtauyzdy + dtauzzdz), (nz-h, ny-2h, nx-2h)
  if (inz) *vz = vz0 - cz * (D2 + D5 + D6);
}

__global__ void __launch_bounds__(256, 5) k3_str_e(const Step3 a) {
  const G3 &g = a.g;
  const Cell3 e = cell3(g, a.shot0, a.nshots, 1);
  if (!e.ok) return;
  const int r = e.r, y = e.y, c = e.c, nz = g.nz, ny = g.ny, nx = g.nx;
  if (r > nz || y > ny || c > nx) return;
  const int64_t so = e.shot * g.fs, o = so + g.S(r, y, c), oc = o - so;
  const int64_t sx = (int64_t)g.NYP * g.NZP, sy = g.NZP;
  const float *vx = a.f[GPI_VX] + so, *vy = a.f[GPI_VY] + so, *vz = a.f[GPI_VZ] + so;
  // every stencil read first (in the padded storage for r, y, c <= n)
  const int64_t b = g.S(r, y, c), bxy = g.S(r + 3, y, c + 3), bxz = g.S(r, y + 3, c + 3), byx = g.S(r + 3, y + 3, c);
  float D9 = st4(vx[b], vx[b + sx], vx[b + 2 * sx], vx[b + 3 * sx]) * a.dxI;            // @d_xa(vx)
  float D10 = st4(vy[b], vy[b + sy], vy[b + 2 * sy], vy[b + 3 * sy]) * a.dyI;           // @d_ya(vy)
  float D11 = st4(vz[b], vz[b + 1], vz[b + 2], vz[b + 3]) * a.dzI;                      // @d_za(vz)
  float D12 = st4(vx[bxy], vx[bxy + sy], vx[bxy + 2 * sy], vx[bxy + 3 * sy]) * a.dyI;   // @d_yi(vx)
  float D14 = st4(vy[byx], vy[byx + sx], vy[byx + 2 * sx], vy[byx + 3 * sx]) * a.dxI;   // @d_xi(vy)
  float D13 = st4(vx[bxz], vx[bxz + 1], vx[bxz + 2], vx[bxz + 3]) * a.dzI;              // @d_zi(vx)
  float D16 = st4(vz[byx], vz[byx + sx], vz[byx + 2 * sx], vz[byx + 3 * sx]) * a.dxI;   // @d_xi(vz)
  float D15 = st4(vy[bxz], vy[bxz + 1], vy[bxz + 2], vy[bxz + 3]) * a.dzI;              // @d_zi(vy)
  float D17 = st4(vz[bxy], vz[bxy + sy], vz[bxy + 2 * sy], vz[bxy + 3 * sy]) * a.dyI;   // @d_yi(vz)
  const float M = a.cf[6][oc], L = a.cf[7][oc], mxz = a.cf[3][oc], mxy = a.cf[4][oc], myz = a.cf[5][oc];
  float *txx = a.f[GPI_TAUXX] + o, *tyy = a.f[GPI_TAUYY] + o, *tzz = a.f[GPI_TAUZZ] + o;
  float *txy = a.f[GPI_TAUXY] + o, *txz = a.f[GPI_TAUXZ] + o, *tyz = a.f[GPI_TAUYZ] + o;
  const float txx0 = *txx, tyy0 = *tyy, tzz0 = *tzz, txy0 = *txy, txz0 = *txz, tyz0 = *tyz;
  const bool ixy = r <= nz - 6 && y <= ny - 3 && c <= nx - 3, ixz = r <= nz - 3 && y <= ny - 6 && c <= nx - 3,
             iyz = r <= nz - 3 && y <= ny - 3 && c <= nx - 6;
  // CPML memory only where a derivative index can fall into a strip
  // (strips of extent-(n-3) .. extent-n derivative fields)
  const int np = a.m.npml;
  if (c <= np || c > nx - 3 - np || y <= np || y > ny - 3 - np || r <= np || r > nz - 3 - np) {
    D9 = mem3(D9, g, a.m, e.shot, 9, 2, c, nx, r, y, c);
    D10 = mem3(D10, g, a.m, e.shot, 10, 1, y, ny, r, y, c);
    D11 = mem3(D11, g, a.m, e.shot, 11, 0, r, nz, r, y, c);
    if (ixy) {
      D12 = mem3(D12, g, a.m, e.shot, 12, 1, y, ny - 3, r, y, c);
      D14 = mem3(D14, g, a.m, e.shot, 14, 2, c, nx - 3, r, y, c);
    }
    if (ixz) {
      D13 = mem3(D13, g, a.m, e.shot, 13, 0, r, nz - 3, r, y, c);
      D16 = mem3(D16, g, a.m, e.shot, 16, 2, c, nx - 3, r, y, c);
    }
    if (iyz) {
      D15 = mem3(D15, g, a.m, e.shot, 15, 0, r, nz - 3, r, y, c);
      D17 = mem3(D17, g, a.m, e.shot, 17, 1, y, ny - 3, r, y, c);
    }
  }
  // compute_stressii!: full grid
  *txx = txx0 - (M * D9) - (L * (D10 + D11));
  *tyy = tyy0 - (M * D10) - (L * (D9 + D11));
  *tzz = tzz0 - (M * D11) - (L * (D10 + D9));
  // tauxy (nz-2h, ny-h, nx-h): -= dtavxyimu (dvxdy + dvydx)
  if (ixy) *txy = txy0 - mxy * (D12 + D14);
  // tauxz (nz-h, ny-2h, nx-h): -= dtavxzimu (dvxdz + dvzdx)
  if (ixz) *txz = txz0 - mxz * (D13 + D16);
  // tauyz (nz-h, ny-h, nx-2h): -= dtavyzimu (dvydz + dvzdy)
  if (iyz) *tyz = tyz0 - myz * (D15 + D17);
}

// free_surface_mirror!(tauzz), free_surface!(tauxz, tauyz) at z = 1
__global__ void k3_free(float *tzz, float *txz, float *tyz, G3 g, int nshots) {
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int c = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int shot = blockIdx.z;
  if (y > g.ny || c > g.nx || shot >= nshots) return;
  const int64_t so = shot * g.fs;
  tzz[so + g.S(1, y, c)] = -tzz[so + g.S(2, y, c)];
  if (y <= g.ny - 6 && c <= g.nx - 3) txz[so + g.S(1, y, c)] = 0.f;
  if (y <= g.ny - 3 && c <= g.nx - 6) tyz[so + g.S(1, y, c)] = 0.f;
}

// one face of dirichlet{x,y,z}{min,max}! (src/fdtd/dirichlet.jl:1-79): the
// other velocity components vanish on the face, the normal component is
// mirrored into the two ghost layers
__global__ void k3_dirichlet(float *vx, float *vy, float *vz, G3 g, int nshots, int axis, int ismax) {
  const int n[3] = {g.nz, g.ny, g.nx};
  const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
  const int ja = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jb = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int shot = blockIdx.z;
  if (ja > n[oa] || jb > n[ob] || shot >= nshots) return;
  const int64_t so = shot * g.fs;
  float *v[3] = {vz + so, vy + so, vx + so};  // by axis
  const int nn = n[axis];
  int idx[3];
  idx[oa] = ja;
  idx[ob] = jb;
  for (int o2 = 0; o2 < 3; o2++) {
    if (o2 == axis) continue;
    idx[axis] = ismax ? nn : 1;
    v[o2][g.S(idx[0], idx[1], idx[2])] = 0.f;
  }
  for (int ifd = 1; ifd <= 2; ifd++) {
    const int gi = ismax ? nn + 4 - ifd : ifd, si = ismax ? nn + ifd - 1 : 5 - ifd;
    int ig[3] = {idx[0], idx[1], idx[2]}, is[3] = {idx[0], idx[1], idx[2]};
    ig[axis] = gi;
    is[axis] = si;
    v[axis][g.S(ig[0], ig[1], ig[2])] = -v[axis][g.S(is[0], is[1], is[2])];
  }
}

// sources of one step: every (shot, kind) group adds its cells' amounts in
// cell order (add_velocity_source! / add_stress_source!, src/fdtd/source.jl)
struct Fields3 {
  float *f[NFIELD];
};
__device__ __forceinline__ void inject_cell(const InjCell &c, float amt, int kind, int64_t so, Fields3 &fld,
                                            int physics) {
  if (kind == 0) fld.f[GPI_VX][so + c.off] = fld.f[GPI_VX][so + c.off] + amt;
  if (kind == 1) fld.f[GPI_VY][so + c.off] = fld.f[GPI_VY][so + c.off] + amt;
  if (kind == 2) fld.f[GPI_VZ][so + c.off] = fld.f[GPI_VZ][so + c.off] + amt;
  if (kind == 3) {
    if (physics == GPI_ACOUSTIC) {
      fld.f[GPI_P][so + c.off] = fld.f[GPI_P][so + c.off] + amt;
    } else {
      fld.f[GPI_TAUXX][so + c.off] = fld.f[GPI_TAUXX][so + c.off] + amt;
      if (fld.f[GPI_TAUYY])  // absent in 2-D (the generic-order steps share this kernel)
        fld.f[GPI_TAUYY][so + c.off] = fld.f[GPI_TAUYY][so + c.off] + amt;
      fld.f[GPI_TAUZZ][so + c.off] = fld.f[GPI_TAUZZ][so + c.off] + amt;
    }
  }
}

// add_stress_source! / add_velocity_source! of one wavefield, one thread per
// (shot, kind) group, cells in order: for groups where two source fields
// reach the same cell (stress sources on several fields)
__global__ void k3_inject_groups(const InjCell *cells, const int32_t *gptr, const float *amount, Fields3 fld,
                                 int64_t fs, int nshots, int velocity, int physics) {
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= nshots * NKIND) return;
  const int shot = gi / NKIND, kind = gi % NKIND;
  if ((kind < 3) != (velocity != 0)) return;
  for (int k = gptr[gi]; k < gptr[gi + 1]; k++) inject_cell(cells[k], amount[k], kind, shot * fs, fld, physics);
}

// the same, one thread per injection cell, when the cells of every group
// are distinct (compile_sources merges the contributions of one source
// field to a cell), so that the adds commute
__global__ void k3_inject(const InjCell *cells, const int32_t *gptr, const float *amount, Fields3 fld, int64_t fs,
                          int nshots, int velocity, int physics) {
  const int ng = nshots * NKIND;
  const int k = gptr[0] + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= gptr[ng]) return;
  // the group of cell k: the last g with gptr[g] <= k
  int lo = 0, hi = ng - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (gptr[mid] <= k)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int shot = lo / NKIND, kind = lo % NKIND;
  if ((kind < 3) != (velocity != 0)) return;
  inject_cell(cells[k], amount[k], kind, shot * fs, fld, physics);
}

// add_velocity_source! (velocity = 1) or add_stress_source! (0) of
// wavefield ipw into its current buffer, from the amounts of this step
int inject_sources(Plan *p, int ipw, int velocity) {
  const int ng = p->d.nshots * NKIND;
  const size_t g0 = (size_t)ipw * ng;
  const int ncw = p->group_ptr.empty() ? 0 : p->group_ptr[g0 + ng] - p->group_ptr[g0];  // cells of this wavefield
  if (ncw <= 0) return GPI_OK;
  Fields3 fl;
  for (int k = 0; k < NFIELD; k++) fl.f[k] = p->state[p->cur[ipw]][ipw][k];
  const int32_t *gptr = p->d_group_ptr + g0;
  if (p->inj_shared)
    k3_inject_groups<<<(ng + 127) / 128, 128, 0, p->stream>>>(p->d_cells, gptr, p->d_amount, fl, p->fstride,
                                                              p->d.nshots, velocity, p->d.physics);
  else
    k3_inject<<<(ncw + 127) / 128, 128, 0, p->stream>>>(p->d_cells, gptr, p->d_amount, fl, p->fstride, p->d.nshots,
                                                        velocity, p->d.physics);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// one step of wavefield ipw (vonly: bit 0 velocity half step only, bit 1
// with the velocity sources)
int step3_wavefield(Plan *p, int ipw, int vonly) {
  const bool ac = p->d.physics == GPI_ACOUSTIC;
  Step3 a;
  a.g = G3{p->d.nz, p->d.ny, p->d.nx, p->NZP, p->NYP, p->fstride};
  a.m.pml = p->pml;
  a.m.npml = p->d.npml;
  a.m.w = 2 * p->d.npml;
  a.m.faces = p->d.pml_faces;
  const int A = p->cur[ipw];  // 3-D steps update in place
  for (int q = 0; q < 18; q++) {
    a.m.psi[q] = q < p->nder ? p->psi[A][ipw][q] : nullptr;
    a.m.pss[q] = q < p->nder ? p->psi_stride[q] : 0;
  }
  Fields3 fl;
  for (int f = 0; f < NFIELD; f++) a.f[f] = fl.f[f] = p->state[A][ipw][f];
  const int32_t *gptr = p->d_group_ptr + (int64_t)ipw * p->d.nshots * NKIND;  // this wavefield's cell groups
  for (int i = 0; i < 8; i++) a.cf[i] = p->coef[i];
  a.dzI = (float)(1.0 / (p->d.dz * 24.0));
  a.dyI = (float)(1.0 / (p->d.dy * 24.0));
  a.dxI = (float)(1.0 / (p->d.dx * 24.0));
  if (p->d.nx + 3 > 65535) return fail(p, GPI_E_UNSUPPORTED, "3-D grids are limited to 65532 columns");
  const dim3 blk(32, 8);
  // the velocity passes cover cells from (4, 4, 4) (their update domains),
  // the stress passes from (1, 1, 1)
  // x-marching launch (acoustic): (z, y) tiles of the cells from `base`,
  // the columns split into runs so that about four waves of blocks start
  auto xm_grid = [&](int base, int nsh, dim3 *g2, int *ncx) -> bool {
    const int nzt = (p->d.nz + 1 - base + XM_Z - 1) / XM_Z, nyt = (p->d.ny + 1 - base + XM_Y - 1) / XM_Y;
    const int tiles = nzt * nyt * nsh;
    *ncx = std::max(1, std::min((p->d.nx + 1 - base) / 16, (4 * 152 * 8 + tiles - 1) / tiles));
    *g2 = dim3(nzt, nyt, *ncx * nsh);
    return (int64_t)*ncx * nsh <= 65535;
  };
  auto pass = [&](bool vel) {
    const int base = vel ? 4 : 1;
    const int nc = p->d.nx + 4 - base;
    const int chunk = 65535 / nc;  // shots per launch (grid z = columns x shots)
    for (int s0 = 0; s0 < p->d.nshots; s0 += chunk) {
      Step3 b = a;
      b.shot0 = s0;
      b.nshots = std::min(chunk, p->d.nshots - s0);
      const dim3 grd((p->d.nz + 4 - base + 31) / 32, (p->d.ny + 4 - base + 7) / 8, nc * b.nshots);
      dim3 g2;
      int ncx = 1;
      const bool xm = ac && xm_grid(base, b.nshots, &g2, &ncx);
      if (vel) {
        if (xm)
          k3_vel_a_xm<<<g2, dim3(XM_Z, XM_Y), 0, p->stream>>>(b, ncx);
        else if (ac)
          k3_vel_a<<<grd, blk, 0, p->stream>>>(b);
        else
          k3_vel_e<<<grd, blk, 0, p->stream>>>(b);
      } else {
        if (xm)
          k3_str_a_xm<<<g2, dim3(XM_Z, XM_Y), 0, p->stream>>>(b, ncx);
        else if (ac)
          k3_str_a<<<grd, blk, 0, p->stream>>>(b);
        else
          k3_str_e<<<grd, blk, 0, p->stream>>>(b);
      }
      p->launches++;
    }
  };

  pass(true);
  // rigid faces in the order x, y, z; min, max (update_v!)
  const int seq[6][2] = {{2, 0}, {2, 1}, {1, 0}, {1, 1}, {0, 0}, {0, 1}};
  const int fmask[3][2] = {{GPI_ZMIN, GPI_ZMAX}, {GPI_YMIN, GPI_YMAX}, {GPI_XMIN, GPI_XMAX}};
  const int n[3] = {p->d.nz, p->d.ny, p->d.nx};
  const int nsz = std::min(p->d.nshots, 65535);
  for (int s = 0; s < 6; s++) {
    const int axis = seq[s][0], ismax = seq[s][1];
    if (!(p->d.rigid_faces & fmask[axis][ismax])) continue;
    const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
    const dim3 db(32, 8), dg((n[oa] + 31) / 32, (n[ob] + 7) / 8, nsz);
    k3_dirichlet<<<dg, db, 0, p->stream>>>(a.f[GPI_VX], a.f[GPI_VY], a.f[GPI_VZ], a.g, p->d.nshots, axis, ismax);
    p->launches++;
  }
  const int ng = p->d.nshots * NKIND;
  const size_t g0 = (size_t)ipw * ng;
  const int ncw = p->group_ptr.empty() ? 0 : p->group_ptr[g0 + ng] - p->group_ptr[g0];  // cells of this wavefield
  auto inject = [&](int velocity) {
    if (p->inj_shared)
      k3_inject_groups<<<(ng + 127) / 128, 128, 0, p->stream>>>(p->d_cells, gptr, p->d_amount, fl, p->fstride,
                                                                p->d.nshots, velocity, p->d.physics);
    else
      k3_inject<<<(ncw + 127) / 128, 128, 0, p->stream>>>(p->d_cells, gptr, p->d_amount, fl, p->fstride,
                                                          p->d.nshots, velocity, p->d.physics);
    p->launches++;
  };
  if ((!vonly || (vonly & 2)) && ncw > 0) inject(1);
  if (vonly) {
    GPI_CUDA(p, cudaGetLastError());
    return GPI_OK;
  }
  pass(false);
  if (!ac && (p->d.free_faces & GPI_ZMIN)) {
    const dim3 fb(32, 8), fg((p->d.nx + 31) / 32, (p->d.ny + 7) / 8, nsz);
    k3_free<<<fg, fb, 0, p->stream>>>(a.f[GPI_TAUZZ], a.f[GPI_TAUXZ], a.f[GPI_TAUYZ], a.g, p->d.nshots);
    p->launches++;
  }
  if (ncw > 0) inject(0);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

int step_acoustic3d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  (void)ipw_mask;
  (void)it;
  (void)mode;
  return step3_wavefield(p, 0, vonly);
}
int step_elastic3d(Plan *p, int ipw_mask, int it, int mode, int vonly) {
  (void)ipw_mask;
  (void)it;
  (void)mode;
  return step3_wavefield(p, 0, vonly);
}

}  // namespace gpi
