// k_generic.cu -- time steps at stencil orders 2, 6 and 8 (2-D and 3-D,
// acoustic and elastic), forward runs.
//
// The reference selects the order of its staggered stencils at compile
// time (set_preferences(order=...), src/GeoPhyInv.jl:69-100; the macros of
// src/fdtd/diff2D.jl and diff3D.jl for orders 2, 4, 6, 8; h = order - 1,
// _fd_npml = 40 + h).  The fused order-4 kernels (k_acoustic2d.cu,
// k_elastic2d.cu, k_3d.cu) carry the order-4 halos in their tiles; the
// other orders run this path, which keeps the reference's structure: per
// step the derivative fields of the stresses (or p) are materialised with
// their CPML memory (update_dstress!), the velocities updated (compute_v!)
// and the rigid faces mirrored (dirichlet*!, src/fdtd/dirichlet.jl:1-79),
// the velocity sources added, then the velocity derivatives (update_dv!),
// the stresses (compute_p! / compute_stress*!, free surface) and the stress
// sources -- one thread per cell of each field, in place, on the plan's
// padded storage (every field and derivative shares the index map, so a
// cell (r, y, c) of any shape sits at the same offset).  Records and source
// amounts come from the aux kernel as in the other paths.
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
__device__ __forceinline__ float gstencil(const float *a, int64_t s) {
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
  GGeo g;
  const float *src;  // shot 0
  float *out;        // shot 0
  int n1, n2, n3;    // derivative extents (z, y, x)
  int oz, oy, ox;    // source offset (inner: h on the other axes)
  int axis;
  float dsI;
  // CPML
  float *psi;  // shot 0 (null: no strip on this axis)
  int64_t pss;
  const float *pa, *pb, *pk;  // profile of this derivative, 2 npml each
  int npml, lo, hi, zsw;
  int nshots;
};

template <int ORDER>
__global__ void __launch_bounds__(256) k_gderiv(const GDer a) {
  const GGeo &g = a.g;
  const int64_t per = (int64_t)a.n1 * a.n2 * a.n3, total = per * a.nshots;
  const int64_t st = a.axis == 0 ? 1 : a.axis == 1 ? (int64_t)g.NZP : (int64_t)g.NYP * g.NZP;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i - shot * per;
    const int iz = (int)(k % a.n1) + 1;
    const int iy = (int)((k / a.n1) % a.n2) + 1;
    const int ix = (int)(k / ((int64_t)a.n1 * a.n2)) + 1;
    const int64_t so = shot * g.fs;
    float D = gstencil<ORDER>(a.src + so + g.S(iz + a.oz, iy + a.oy, ix + a.ox), st) * a.dsI;
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
    a.out[so + g.S(iz, iy, ix)] = D;
  }
}

// compute_v!: @inn(v) += c * D (acoustic, advance_acou.jl:273-284) or
// -= c * (D1 + D2 [+ D3]) (elastic, advance_elastic.jl:69-110), the
// coefficient stored at the velocity cell
struct GVel {
  GGeo g;
  float *v;  // shot 0
  const float *cf;
  const float *d1, *d2, *d3;  // derivatives at the @all index (d2, d3 null where absent)
  int r1, r2, r3, hy;         // @inn extents and the y offset (0 in 2-D)
  int elastic, nshots;
};
__global__ void __launch_bounds__(256) k_gvel(const GVel a) {
  const GGeo &g = a.g;
  const int64_t per = (int64_t)a.r1 * a.r2 * a.r3, total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i - shot * per;
    const int iz = (int)(k % a.r1) + 1;
    const int iy = (int)((k / a.r1) % a.r2) + 1;
    const int ix = (int)(k / ((int64_t)a.r1 * a.r2)) + 1;
    const int64_t so = shot * g.fs, od = so + g.S(iz, iy, ix);
    const int64_t ov = g.S(iz + g.h, iy + a.hy, ix + g.h);
    const float c = a.cf[ov];
    float *v = a.v + so + ov;
    if (!a.elastic) {
      *v = *v + c * a.d1[od];
    } else if (!a.d3) {
      *v = *v - c * (a.d1[od] + a.d2[od]);
    } else {
      *v = *v - c * (a.d1[od] + a.d2[od] + a.d3[od]);
    }
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
  float *f[NFIELD];            // shot 0
  const float *cf[8];          // coefficients
  const float *d[18];          // derivatives
  int elastic, nshots, free_zmin;
};
__global__ void __launch_bounds__(256) k_gstress_a(const GStr a) {
  const GGeo &g = a.g;
  const int n2 = g.ndim == 3 ? g.ny : 1;
  const int64_t per = (int64_t)g.nz * n2 * g.nx, total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i - shot * per;
    const int r = (int)(k % g.nz) + 1, y = (int)((k / g.nz) % n2) + 1, c = (int)(k / ((int64_t)g.nz * n2)) + 1;
    const int64_t o = g.S(r, y, c), so = shot * g.fs;
    float *p = a.f[GPI_P] + so + o;
    if (g.ndim == 3)  // (dvxdx + dvzdz + dvydy) * dtK
      *p = *p + (a.d[3][so + o] + a.d[5][so + o] + a.d[4][so + o]) * a.cf[3][o];
    else
      *p = *p + (a.d[2][so + o] + a.d[3][so + o]) * a.cf[2][o];
  }
}

// compute_stressii! / compute_stressij! (advance_elastic.jl:155-213): the
// normal stresses over their (full) shape, each shear stress over its own
__global__ void __launch_bounds__(256) k_gstress_e(const GStr a) {
  const GGeo &g = a.g;
  const int h = g.h, three = g.ndim == 3;
  const int n2 = three ? g.ny : 1;
  const int64_t per = (int64_t)g.nz * n2 * g.nx, total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i - shot * per;
    const int r = (int)(k % g.nz) + 1, y = (int)((k / g.nz) % n2) + 1, c = (int)(k / ((int64_t)g.nz * n2)) + 1;
    const int64_t o = g.S(r, y, c), so = shot * g.fs, x = so + o;
    if (!three) {
      const float M = a.cf[3][o], L = a.cf[4][o];
      const float dvxdx = a.d[4][x], dvzdz = a.d[5][x];
      float *txx = a.f[GPI_TAUXX] + x, *tzz = a.f[GPI_TAUZZ] + x;
      *txx = *txx - (M * dvxdx) - (L * (dvzdz));
      *tzz = *tzz - (M * dvzdz) - (L * (dvxdx));
      if (r <= g.nz - h && c <= g.nx - h) {  // tauxz (n-h, n-h)
        float *txz = a.f[GPI_TAUXZ] + x;
        *txz = *txz - a.cf[2][o] * (a.d[6][x] + a.d[7][x]);
      }
    } else {
      const float M = a.cf[6][o], L = a.cf[7][o];
      const float dvxdx = a.d[9][x], dvydy = a.d[10][x], dvzdz = a.d[11][x];
      float *txx = a.f[GPI_TAUXX] + x, *tyy = a.f[GPI_TAUYY] + x, *tzz = a.f[GPI_TAUZZ] + x;
      *txx = *txx - (M * dvxdx) - (L * (dvydy + dvzdz));
      *tyy = *tyy - (M * dvydy) - (L * (dvxdx + dvzdz));
      *tzz = *tzz - (M * dvzdz) - (L * (dvydy + dvxdx));
      if (r <= g.nz - h && y <= g.ny - 2 * h && c <= g.nx - h) {  // tauxz (n-h, n-2h, n-h)
        float *t = a.f[GPI_TAUXZ] + x;
        *t = *t - a.cf[3][o] * (a.d[13][x] + a.d[16][x]);
      }
      if (r <= g.nz - 2 * h && y <= g.ny - h && c <= g.nx - h) {  // tauxy (n-2h, n-h, n-h)
        float *t = a.f[GPI_TAUXY] + x;
        *t = *t - a.cf[4][o] * (a.d[12][x] + a.d[14][x]);
      }
      if (r <= g.nz - h && y <= g.ny - h && c <= g.nx - 2 * h) {  // tauyz (n-h, n-h, n-2h)
        float *t = a.f[GPI_TAUYZ] + x;
        *t = *t - a.cf[5][o] * (a.d[15][x] + a.d[17][x]);
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
  const int grid = 152 * 16;
  auto derivs = [&](int q0, int q1) -> int {
    for (int q = q0; q < q1; q++) {
      const GSpec &s = spec[q];
      GDer a;
      a.g = g;
      a.src = f[s.src];
      a.out = p->der[q];
      a.n1 = gext(s.kz, n[0], h);
      a.n2 = three ? gext(s.ky, n[1], h) : 1;
      a.n3 = gext(s.kx, n[2], h);
      a.oz = s.inner && s.axis != 0 ? h : 0;
      a.oy = three && s.inner && s.axis != 1 ? h : 0;
      a.ox = s.inner && s.axis != 2 ? h : 0;
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
      a.nshots = p->d.nshots;
      k_gderiv<ORDER><<<grid, 256, 0, p->stream>>>(a);
      p->launches++;
    }
    GPI_CUDA(p, cudaGetLastError());
    return GPI_OK;
  };
  // update_dstress! + compute_v!
  if (int rc = derivs(0, nstress)) return rc;
  const int vid[3] = {GPI_VX, GPI_VY, GPI_VZ};
  for (int q = 0; q < 3; q++) {
    if (q == 1 && !three) continue;
    GVel a;
    a.g = g;
    a.v = f[vid[q]];
    a.cf = p->coef[q == 0 ? 0 : q == 1 ? 1 : (three ? 2 : 1)];
    int kz, ky, kx;
    field_kinds(vid[q], &kz, &ky, &kx);
    a.r1 = nkind(kz, n[0], h) - 2 * h;
    a.r2 = three ? nkind(ky, n[1], h) - 2 * h : 1;
    a.r3 = nkind(kx, n[2], h) - 2 * h;
    a.hy = three ? h : 0;
    a.elastic = !ac;
    a.nshots = p->d.nshots;
    a.d2 = a.d3 = nullptr;
    if (ac) {
      a.d1 = p->der[three ? q : (q == 0 ? 0 : 1)];
    } else if (!three) {
      a.d1 = p->der[q == 0 ? 0 : 1];
      a.d2 = p->der[q == 0 ? 3 : 2];
    } else {
      const int i3[3][3] = {{0, 4, 8}, {1, 3, 7}, {2, 5, 6}};
      a.d1 = p->der[i3[q][0]];
      a.d2 = p->der[i3[q][1]];
      a.d3 = p->der[i3[q][2]];
    }
    k_gvel<<<grid, 256, 0, p->stream>>>(a);
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
  if (int rc = derivs(nstress, nder)) return rc;
  GStr a;
  a.g = g;
  for (int k = 0; k < NFIELD; k++) a.f[k] = f[k];
  for (int k = 0; k < 8; k++) a.cf[k] = p->coef[k];
  for (int k = 0; k < 18; k++) a.d[k] = p->der[k];
  a.elastic = !ac;
  a.nshots = p->d.nshots;
  a.free_zmin = (p->d.free_faces & GPI_ZMIN) != 0;
  if (ac)
    k_gstress_a<<<grid, 256, 0, p->stream>>>(a);
  else
    k_gstress_e<<<grid, 256, 0, p->stream>>>(a);
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
