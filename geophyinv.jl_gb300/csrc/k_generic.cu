// k_generic.cu -- time steps at stencil orders 2, 6 and 8 (2-D and 3-D,
// acoustic and elastic), forward runs.
//
// The reference selects the order of its staggered stencils at compile
// time (set_preferences(order=...), src/GeoPhyInv.jl:69-100; the macros of
// src/fdtd/diff2D.jl and diff3D.jl for orders 2, 4, 6, 8; h = order - 1,
// _fd_npml = 40 + h).  The fused order-4 kernels (k_acoustic2d.cu,
// k_elastic2d.cu, k_3d.cu) carry the order-4 halos in their tiles; the
// other orders run this path, which keeps the reference's structure: per
// step the velocities are updated (compute_v!) from the derivatives of the
// stresses (or p) with their CPML memory (update_dstress!), the rigid faces
// mirrored (dirichlet*!, src/fdtd/dirichlet.jl:1-79), the velocity sources
// added, then the stresses (compute_p! / compute_stress*!) from the
// velocity derivatives (update_dv!), the free surface and the stress
// sources -- one thread per cell of each updated field, in place, on the
// plan's padded storage (every field shares the index map, so a cell
// (r, y, c) of any shape sits at the same offset).  The reference
// materialises each derivative field; here the thread that consumes a
// derivative cell computes it in registers: the derivative shapes equal
// the update domains that read them (the @inn domain of a velocity, the
// shape of a stress), so every derivative cell, and its CPML memory, is
// still evaluated exactly once per step, with the same arithmetic.
// Records and source amounts come from the aux kernel as in the other
// paths.
//
// The derivative table restates the reference's (src/fdtd/advance_acou.jl:
// 258-299, src/fdtd/advance_elastic.jl:10-153, src/fields.jl:92-671):
// derivative q of shape kinds (kz, ky, kx) along `axis` of field `src`,
// @d_?a reading the source at the derivative's own index, @d_?i ("inner")
// at +h on the other two axes.
#include <algorithm>

#include "k_stencil.cuh"

namespace gpi {

namespace {

enum { GKF = 0, GKV = 1, GKH = 2, GKI = 3 };  // shape kinds n, n+h, n-h, n-2h

struct GSpec {
  int axis, kz, ky, kx, src, inner;
};
// (the canonical derivative order of the engine and its oracle)
const GSpec GA2[4] = {{2, GKI, GKF, GKH, GPI_P, 1},
                      {0, GKH, GKF, GKI, GPI_P, 1},
                      {2, GKF, GKF, GKF, GPI_VX, 0},
                      {0, GKF, GKF, GKF, GPI_VZ, 0}};
const GSpec GE2[8] = {{2, GKI, GKF, GKH, GPI_TAUXX, 1}, {2, GKH, GKF, GKI, GPI_TAUXZ, 0},
                      {0, GKH, GKF, GKI, GPI_TAUZZ, 1}, {0, GKI, GKF, GKH, GPI_TAUXZ, 0},
                      {2, GKF, GKF, GKF, GPI_VX, 0},    {0, GKF, GKF, GKF, GPI_VZ, 0},
                      {0, GKH, GKF, GKH, GPI_VX, 1},    {2, GKH, GKF, GKH, GPI_VZ, 1}};
const GSpec GA3[6] = {{2, GKI, GKI, GKH, GPI_P, 1},  {1, GKI, GKH, GKI, GPI_P, 1},  {0, GKH, GKI, GKI, GPI_P, 1},
                      {2, GKF, GKF, GKF, GPI_VX, 0}, {1, GKF, GKF, GKF, GPI_VY, 0}, {0, GKF, GKF, GKF, GPI_VZ, 0}};
const GSpec GE3[18] = {{2, GKI, GKI, GKH, GPI_TAUXX, 1}, {2, GKI, GKH, GKI, GPI_TAUXY, 0},
                       {2, GKH, GKI, GKI, GPI_TAUXZ, 0}, {1, GKI, GKH, GKI, GPI_TAUYY, 1},
                       {1, GKI, GKI, GKH, GPI_TAUXY, 0}, {1, GKH, GKI, GKI, GPI_TAUYZ, 0},
                       {0, GKH, GKI, GKI, GPI_TAUZZ, 1}, {0, GKI, GKH, GKI, GPI_TAUYZ, 0},
                       {0, GKI, GKI, GKH, GPI_TAUXZ, 0}, {2, GKF, GKF, GKF, GPI_VX, 0},
                       {1, GKF, GKF, GKF, GPI_VY, 0},    {0, GKF, GKF, GKF, GPI_VZ, 0},
                       {1, GKI, GKH, GKH, GPI_VX, 1},    {0, GKH, GKI, GKH, GPI_VX, 1},
                       {2, GKI, GKH, GKH, GPI_VY, 1},    {0, GKH, GKH, GKI, GPI_VY, 1},
                       {2, GKH, GKI, GKH, GPI_VZ, 1},    {1, GKH, GKH, GKI, GPI_VZ, 1}};

int gext(int kind, int n, int h) { return kind == GKV ? n + h : kind == GKH ? n - h : kind == GKI ? n - 2 * h : n; }

}  // namespace

// geometry of the padded storage (2-D: one y plane)
struct GGeo {
  int nz, ny, nx, NZP, NYP, ndim, h;
  int64_t fs;
  __device__ __forceinline__ int64_t S(int r, int y, int c) const {
    return ((int64_t)(c - 1 + XOFF) * NYP + (ndim == 3 ? (y - 1 + YOFF) : 0)) * NZP + (r - 1 + ZOFF);
  }
};

// staggered difference of order ORDER along stride s (src/fdtd/diff2D.jl,
// diff3D.jl: @d_?a / @d_?i), the reference's coefficients and sum order
template <int ORDER>
__device__ __forceinline__ float gstencil(const float *a, int s) {
  if constexpr (ORDER == 2) {
    return a[s] - a[0];
  } else if constexpr (ORDER == 4) {
    return a[2 * s] * 27.0f - a[s] * 27.0f + a[0] - a[3 * s];
  } else if constexpr (ORDER == 6) {
    return a[3 * s] * 2250.0f - a[2 * s] * 2250.0f + a[s] * 125.0f - a[4 * s] * 125.0f + a[5 * s] * 9.0f -
           a[0] * 9.0f;
  } else {
    return a[4 * s] * 128625.0f - a[3 * s] * 128625.0f + a[2 * s] * 8575.0f - a[5 * s] * 8575.0f +
           a[6 * s] * 1029.0f - a[s] * 1029.0f + a[0] * 75.0f - a[7 * s] * 75.0f;
  }
}

// one derivative field: D = @d(src) * dsI over its shape, with the CPML
// memory on the strips of its axis (memory{x,y,z}!, src/fdtd/cpml.jl:158-215)
struct GDer {
  const float *src;  // shot 0
  int n1, n2, n3;    // derivative extents (z, y, x)
  int soff, st;      // storage offset of the source cell from the derivative
                     // cell (inner: h on the other axes); stride of the axis
  int axis;
  float dsI;
  // CPML
  float *psi;  // shot 0 (null: no strip on this axis)
  int64_t pss;
  const float *pa, *pb, *pk;  // profile of this derivative, 2 npml each
  int npml, lo, hi, zsw;
};

// derivative cell (iz, iy, ix) of shot `shot` at storage offset `base`
// (shot included), its CPML memory advanced
template <int ORDER>
__device__ __forceinline__ float gder_at(const GGeo &g, const GDer &a, int64_t base, int shot, int iz, int iy, int ix) {
  float D = gstencil<ORDER>(a.src + base + a.soff, a.st) * a.dsI;
  if (a.psi) {
    const int ia = a.axis == 0 ? iz : a.axis == 1 ? iy : ix, nd = a.axis == 0 ? a.n1 : a.axis == 1 ? a.n2 : a.n3;
    const int j = pml_slot(ia, nd, a.npml, a.lo, a.hi);
    if (j >= 0) {
      int64_t pi;
      if (g.ndim == 2)
        pi = a.axis == 2 ? (int64_t)j * g.NZP + (iz + ZOFF - 1) : (int64_t)(ix + XOFF - 1) * a.zsw + j;
      else if (a.axis == 2)
        pi = ((int64_t)j * g.NYP + (iy + YOFF - 1)) * g.NZP + (iz + ZOFF - 1);
      else if (a.axis == 1)
        pi = ((int64_t)(ix + XOFF - 1) * (2 * a.npml) + j) * g.NZP + (iz + ZOFF - 1);
      else
        pi = ((int64_t)(ix + XOFF - 1) * g.NYP + (iy + YOFF - 1)) * (2 * a.npml) + j;
      float *ps = a.psi + shot * a.pss + pi;
      const float psi = a.pb[j] * *ps + a.pa[j] * D;
      *ps = psi;
      D = D * a.pk[j] + psi;
    }
  }
  return D;
}

// compute_v!: @inn(v) += c * D (acoustic, advance_acou.jl:273-284) or
// -= c * (D1 + D2 [+ D3]) (elastic, advance_elastic.jl:69-110), the
// coefficient stored at the velocity cell; the derivatives of a component
// share its @inn extents.  One thread updates every component whose domain
// holds its cell (the components read the stresses only, so their order is
// free), so the stress columns two components read come from L1.
struct GVelC {
  float *v;  // shot 0
  const float *cf;
  GDer d[3];  // nd of them
  int nd, r1, r2, r3;
};
struct GVel {
  GGeo g;
  GVelC c[3];  // nc of them
  int nc, hy, elastic;
};
// Launch shape of the per-cell kernels: GT threads along z, grid (the y-x
// columns, z blocks, shots), so that a thread finds its cell without a
// division.
constexpr int GT = 128;
template <int ORDER>
__device__ __forceinline__ void gvel_one(const GGeo &g, const GVelC &a, int hy, int elastic, int shot, int iz, int iy,
                                         int ix) {
  const int64_t ov = g.S(iz + g.h, iy + hy, ix + g.h), od = shot * g.fs + g.S(iz, iy, ix);
  const float c = a.cf[ov];
  float *v = a.v + shot * g.fs + ov;
  const float D1 = gder_at<ORDER>(g, a.d[0], od, shot, iz, iy, ix);
  if (!elastic) {
    *v = *v + c * D1;
  } else if (a.nd == 2) {
    const float D2 = gder_at<ORDER>(g, a.d[1], od, shot, iz, iy, ix);
    *v = *v - c * (D1 + D2);
  } else {
    const float D2 = gder_at<ORDER>(g, a.d[1], od, shot, iz, iy, ix);
    const float D3 = gder_at<ORDER>(g, a.d[2], od, shot, iz, iy, ix);
    *v = *v - c * (D1 + D2 + D3);
  }
}
// grid over the union of the components' domains (r2u columns per x)
template <int ORDER>
__global__ void __launch_bounds__(GT) k_gvel(const GVel a, int r1u, int r2u) {
  const GGeo &g = a.g;
  const int iz = blockIdx.y * GT + threadIdx.x + 1;
  if (iz > r1u) return;
  const bool flat = g.ndim == 2;  // one y plane: the column index is x
  const int iy = flat ? 1 : (int)(blockIdx.x % (unsigned)r2u) + 1;
  const int ix = flat ? (int)blockIdx.x + 1 : (int)(blockIdx.x / (unsigned)r2u) + 1;
  const int shot = blockIdx.z;
  for (int q = 0; q < a.nc; q++) {
    const GVelC &c = a.c[q];
    if (iz <= c.r1 && iy <= c.r2 && ix <= c.r3) gvel_one<ORDER>(g, c, a.hy, a.elastic, shot, iz, iy, ix);
  }
}

// dirichlet{z,y,x}{min,max}! of one face (src/fdtd/dirichlet.jl:1-79): the
// other velocity components vanish at the face, and the face-normal one is
// mirrored onto its order/2 ghost cells
template <int ORDER>
__global__ void k_gdirichlet(float *vz, float *vy, float *vx, GGeo g, int nshots, int axis, int ismax) {
  const int n[3] = {g.nz, g.ny, g.nx};
  const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
  const int na = (oa == 1 && g.ndim == 2) ? 1 : n[oa], nb = n[ob];
  const int ja = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jb = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int shot = blockIdx.z;
  if (ja > na || jb > nb || shot >= nshots) return;
  const int64_t so = shot * g.fs;
  float *v[3] = {vz ? vz + so : nullptr, vy ? vy + so : nullptr, vx ? vx + so : nullptr};  // by axis
  const int nn = n[axis];
  int idx[3] = {1, 1, 1};
  idx[oa] = ja;
  idx[ob] = jb;
  for (int o2 = 0; o2 < 3; o2++) {
    if (o2 == axis || !v[o2]) continue;
    int j[3] = {idx[0], idx[1], idx[2]};
    j[axis] = ismax ? nn : 1;
    v[o2][g.S(j[0], j[1], j[2])] = 0.f;
  }
  for (int ifd = 1; ifd <= ORDER / 2; ifd++) {
    const int gi = ismax ? nn + ORDER - ifd : ifd, si = ismax ? nn + ifd - 1 : ORDER + 1 - ifd;
    int ig[3] = {idx[0], idx[1], idx[2]}, is[3] = {idx[0], idx[1], idx[2]};
    ig[axis] = gi;
    is[axis] = si;
    v[axis][g.S(ig[0], ig[1], ig[2])] = -v[axis][g.S(is[0], is[1], is[2])];
  }
}

// compute_p! (advance_acou.jl:303-313) over every p cell
struct GStr {
  GGeo g;
  float *f[NFIELD];    // shot 0
  const float *cf[8];  // coefficients
  GDer d[9];           // the velocity derivatives, in the canonical order
  int elastic, nshots, free_zmin;
};
template <int ORDER>
__global__ void __launch_bounds__(GT) k_gstress_a(const GStr a) {
  const GGeo &g = a.g;
  const unsigned n2 = g.ndim == 3 ? g.ny : 1;
  const int r = blockIdx.y * GT + threadIdx.x + 1;
  if (r > g.nz) return;
  const int y = n2 == 1 ? 1 : (int)(blockIdx.x % n2) + 1, c = n2 == 1 ? (int)blockIdx.x + 1 : (int)(blockIdx.x / n2) + 1;
  const int shot = blockIdx.z;
  {
    const int64_t o = g.S(r, y, c), so = shot * g.fs, x = so + o;
    float *p = a.f[GPI_P] + x;
    if (g.ndim == 3) {  // (dvxdx + dvzdz + dvydy) * dtK
      const float dx = gder_at<ORDER>(g, a.d[0], x, shot, r, y, c), dy = gder_at<ORDER>(g, a.d[1], x, shot, r, y, c),
                  dz = gder_at<ORDER>(g, a.d[2], x, shot, r, y, c);
      *p = *p + (dx + dz + dy) * a.cf[3][o];
    } else {
      const float dx = gder_at<ORDER>(g, a.d[0], x, shot, r, 1, c), dz = gder_at<ORDER>(g, a.d[1], x, shot, r, 1, c);
      *p = *p + (dx + dz) * a.cf[2][o];
    }
  }
}

// compute_stressii! / compute_stressij! (advance_elastic.jl:155-213): the
// normal stresses over their (full) shape, each shear stress over its own
// (the shape of the two derivatives it reads)
template <int ORDER>
__global__ void __launch_bounds__(GT) k_gstress_e(const GStr a) {
  const GGeo &g = a.g;
  const int h = g.h, three = g.ndim == 3;
  const unsigned n2 = three ? g.ny : 1;
  const int r = blockIdx.y * GT + threadIdx.x + 1;
  if (r > g.nz) return;
  const int y = n2 == 1 ? 1 : (int)(blockIdx.x % n2) + 1, c = n2 == 1 ? (int)blockIdx.x + 1 : (int)(blockIdx.x / n2) + 1;
  const int shot = blockIdx.z;
  {
    const int64_t o = g.S(r, y, c), so = shot * g.fs, x = so + o;
    if (!three) {
      const float M = a.cf[3][o], L = a.cf[4][o];
      const float dvxdx = gder_at<ORDER>(g, a.d[0], x, shot, r, 1, c), dvzdz = gder_at<ORDER>(g, a.d[1], x, shot, r, 1, c);
      float *txx = a.f[GPI_TAUXX] + x, *tzz = a.f[GPI_TAUZZ] + x;
      *txx = *txx - (M * dvxdx) - (L * (dvzdz));
      *tzz = *tzz - (M * dvzdz) - (L * (dvxdx));
      if (r <= g.nz - h && c <= g.nx - h) {  // tauxz (n-h, n-h)
        const float dvxdz = gder_at<ORDER>(g, a.d[2], x, shot, r, 1, c), dvzdx = gder_at<ORDER>(g, a.d[3], x, shot, r, 1, c);
        float *txz = a.f[GPI_TAUXZ] + x;
        *txz = *txz - a.cf[2][o] * (dvxdz + dvzdx);
      }
    } else {
      const float M = a.cf[6][o], L = a.cf[7][o];
      const float dvxdx = gder_at<ORDER>(g, a.d[0], x, shot, r, y, c), dvydy = gder_at<ORDER>(g, a.d[1], x, shot, r, y, c),
                  dvzdz = gder_at<ORDER>(g, a.d[2], x, shot, r, y, c);
      float *txx = a.f[GPI_TAUXX] + x, *tyy = a.f[GPI_TAUYY] + x, *tzz = a.f[GPI_TAUZZ] + x;
      *txx = *txx - (M * dvxdx) - (L * (dvydy + dvzdz));
      *tyy = *tyy - (M * dvydy) - (L * (dvxdx + dvzdz));
      *tzz = *tzz - (M * dvzdz) - (L * (dvydy + dvxdx));
      if (r <= g.nz - h && y <= g.ny - 2 * h && c <= g.nx - h) {  // tauxz (n-h, n-2h, n-h)
        const float d1 = gder_at<ORDER>(g, a.d[4], x, shot, r, y, c), d2 = gder_at<ORDER>(g, a.d[7], x, shot, r, y, c);
        float *t = a.f[GPI_TAUXZ] + x;
        *t = *t - a.cf[3][o] * (d1 + d2);
      }
      if (r <= g.nz - 2 * h && y <= g.ny - h && c <= g.nx - h) {  // tauxy (n-2h, n-h, n-h)
        const float d1 = gder_at<ORDER>(g, a.d[3], x, shot, r, y, c), d2 = gder_at<ORDER>(g, a.d[5], x, shot, r, y, c);
        float *t = a.f[GPI_TAUXY] + x;
        *t = *t - a.cf[4][o] * (d1 + d2);
      }
      if (r <= g.nz - h && y <= g.ny - h && c <= g.nx - 2 * h) {  // tauyz (n-h, n-h, n-2h)
        const float d1 = gder_at<ORDER>(g, a.d[6], x, shot, r, y, c), d2 = gder_at<ORDER>(g, a.d[8], x, shot, r, y, c);
        float *t = a.f[GPI_TAUYZ] + x;
        *t = *t - a.cf[5][o] * (d1 + d2);
      }
    }
  }
}

// free_surface_mirror!(tauzz), free_surface!(tauxz[, tauyz]) at z = 1
// (advance_elastic.jl:215-230)
__global__ void k_gfree(float *tzz, float *txz, float *tyz, GGeo g, int nshots) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int shot = blockIdx.z;
  const int h = g.h, three = g.ndim == 3;
  if (c > g.nx || y > (three ? g.ny : 1) || shot >= nshots) return;
  const int64_t so = shot * g.fs;
  tzz[so + g.S(1, y, c)] = -tzz[so + g.S(2, y, c)];
  if (!three) {
    if (c <= g.nx - h) txz[so + g.S(1, y, c)] = 0.f;
  } else {
    if (y <= g.ny - 2 * h && c <= g.nx - h) txz[so + g.S(1, y, c)] = 0.f;
    if (y <= g.ny - h && c <= g.nx - 2 * h) tyz[so + g.S(1, y, c)] = 0.f;
  }
}

int inject_sources(Plan *p, int ipw, int velocity);  // k_3d.cu

// one step (vonly: the velocity half step, bit 1 with the velocity sources)
// of wavefield 0 at a stencil order other than 4
template <int ORDER>
static int gstep_order(Plan *p, int vonly) {
  const bool ac = p->d.physics == GPI_ACOUSTIC, three = p->d.ndim == 3;
  const int h = p->h;
  const GGeo g{p->d.nz, p->d.ny, p->d.nx, p->NZP, p->NYP, p->d.ndim, h, p->fstride};
  float *const *f = p->state[p->cur[0]][0];
  const GSpec *spec = ac ? (three ? GA3 : GA2) : (three ? GE3 : GE2);
  const int nder = ac ? (three ? 6 : 4) : (three ? 18 : 8);
  const int nstress = ac ? p->d.ndim : (three ? 9 : 4);
  const int n[3] = {p->d.nz, p->d.ny, p->d.nx};
  const float dsI[3] = {p->gdsI[0], p->gdsI[1], p->gdsI[2]};
  const int fmin[3] = {GPI_ZMIN, GPI_YMIN, GPI_XMIN}, fmax[3] = {GPI_ZMAX, GPI_YMAX, GPI_XMAX};
  auto der = [&](int q) {
    const GSpec &s = spec[q];
    GDer a;
    a.src = f[s.src];
    a.n1 = gext(s.kz, n[0], h);
    a.n2 = three ? gext(s.ky, n[1], h) : 1;
    a.n3 = gext(s.kx, n[2], h);
    const int oz = s.inner && s.axis != 0 ? h : 0, oy = three && s.inner && s.axis != 1 ? h : 0,
              ox = s.inner && s.axis != 2 ? h : 0;
    a.soff = (int)(oz + (int64_t)oy * p->NZP + (int64_t)ox * p->NYP * p->NZP);
    a.st = s.axis == 0 ? 1 : s.axis == 1 ? p->NZP : p->NYP * p->NZP;
    a.axis = s.axis;
    a.dsI = dsI[s.axis];
    a.psi = p->psi[0][0][q];
    a.pss = p->psi_stride[q];
    const int P = 2 * p->d.npml;
    a.pa = p->pml + (int64_t)q * 3 * P;
    a.pb = a.pa + P;
    a.pk = a.pb + P;
    a.npml = p->d.npml;
    a.lo = (p->d.pml_faces & fmin[s.axis]) != 0;
    a.hi = (p->d.pml_faces & fmax[s.axis]) != 0;
    a.zsw = p->zsw;
    return a;
  };
  // update_dstress! + compute_v!
  const int vid[3] = {GPI_VX, GPI_VY, GPI_VZ};
  {
    GVel a;
    a.g = g;
    a.hy = three ? h : 0;
    a.elastic = !ac;
    a.nc = 0;
    int r1u = 0, r2u = 0, r3u = 0;
    for (int q = 0; q < 3; q++) {
      if (q == 1 && !three) continue;
      GVelC &c = a.c[a.nc++];
      c.v = f[vid[q]];
      c.cf = p->coef[q == 0 ? 0 : q == 1 ? 1 : (three ? 2 : 1)];
      int kz, ky, kx;
      field_kinds(vid[q], &kz, &ky, &kx);
      c.r1 = nkind(kz, n[0], h) - 2 * h;
      c.r2 = three ? nkind(ky, n[1], h) - 2 * h : 1;
      c.r3 = nkind(kx, n[2], h) - 2 * h;
      r1u = std::max(r1u, c.r1);
      r2u = std::max(r2u, c.r2);
      r3u = std::max(r3u, c.r3);
      if (ac) {
        c.nd = 1;
        c.d[0] = der(three ? q : (q == 0 ? 0 : 1));
      } else if (!three) {
        c.nd = 2;
        c.d[0] = der(q == 0 ? 0 : 1);
        c.d[1] = der(q == 0 ? 3 : 2);
      } else {
        const int i3[3][3] = {{0, 4, 8}, {1, 3, 7}, {2, 5, 6}};
        c.nd = 3;
        for (int k = 0; k < 3; k++) c.d[k] = der(i3[q][k]);
      }
    }
    const dim3 vg((unsigned)(r2u * r3u), (r1u + GT - 1) / GT, p->d.nshots);
    k_gvel<ORDER><<<vg, GT, 0, p->stream>>>(a, r1u, r2u);
    p->launches++;
  }
  // rigid faces in the order x, y, z; min, max (update_v!)
  const int seq[6][2] = {{2, 0}, {2, 1}, {1, 0}, {1, 1}, {0, 0}, {0, 1}};
  const int nsz = std::min(p->d.nshots, 65535);
  for (int s = 0; s < 6; s++) {
    const int axis = seq[s][0], ismax = seq[s][1];
    if (axis == 1 && !three) continue;
    if (!(p->d.rigid_faces & (ismax ? fmax[axis] : fmin[axis]))) continue;
    const int oa = axis == 0 ? 1 : 0, ob = axis == 2 ? 1 : 2;
    const int na = (oa == 1 && !three) ? 1 : n[oa];
    const dim3 db(32, 8), dg((na + 31) / 32, (n[ob] + 7) / 8, nsz);
    k_gdirichlet<ORDER><<<dg, db, 0, p->stream>>>(f[GPI_VZ], three ? f[GPI_VY] : nullptr, f[GPI_VX], g,
                                                  p->d.nshots, axis, ismax);
    p->launches++;
  }
  GPI_CUDA(p, cudaGetLastError());
  if (!vonly || (vonly & 2))
    if (int rc = inject_sources(p, 0, 1)) return rc;
  if (vonly) return GPI_OK;
  // update_dv! + compute_stress
  GStr a;
  a.g = g;
  for (int k = 0; k < NFIELD; k++) a.f[k] = f[k];
  for (int k = 0; k < 8; k++) a.cf[k] = p->coef[k];
  for (int k = 0; k < nder - nstress; k++) a.d[k] = der(nstress + k);
  a.elastic = !ac;
  a.nshots = p->d.nshots;
  a.free_zmin = (p->d.free_faces & GPI_ZMIN) != 0;
  const dim3 sg((unsigned)((three ? n[1] : 1) * n[2]), (n[0] + GT - 1) / GT, p->d.nshots);
  if (ac)
    k_gstress_a<ORDER><<<sg, GT, 0, p->stream>>>(a);
  else
    k_gstress_e<ORDER><<<sg, GT, 0, p->stream>>>(a);
  p->launches++;
  if (!ac && a.free_zmin) {
    const dim3 fb(32, 8), fg((n[2] + 31) / 32, three ? (n[1] + 7) / 8 : 1, nsz);
    k_gfree<<<fg, fb, 0, p->stream>>>(f[GPI_TAUZZ], f[GPI_TAUXZ], three ? f[GPI_TAUYZ] : nullptr, g, p->d.nshots);
    p->launches++;
  }
  GPI_CUDA(p, cudaGetLastError());
  return inject_sources(p, 0, 0);
}

int step_generic(Plan *p, int vonly) {
  switch (p->d.order) {
    case 2: return gstep_order<2>(p, vonly);
    case 6: return gstep_order<6>(p, vonly);
    case 8: return gstep_order<8>(p, vonly);
    default: return gstep_order<4>(p, vonly);
  }
}

}  // namespace gpi
