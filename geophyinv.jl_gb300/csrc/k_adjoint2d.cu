// k_adjoint2d.cu -- adjoint time step and imaging condition, 2-D acoustic.
//
// One adjoint step (mod_x_proc! with npw = 2, src/fdtd/propagate.jl:138-261):
//   save_tp! of both wavefields (src/fdtd/save_tp.jl:5-14)       -- implicit:
//       the step reads buffer A and writes buffer B, A is the "tp" copy
//   boundary_force! on wavefield 1 (src/fdtd/boundary.jl:113-170) -- done by
//       boundary_io before this call; the replaced strip values are kept in
//       Plan::bprev, since the imaging condition uses the unforced field
//   update of wavefield 1 (time reversal) and of wavefield 2 (adjoint, fed
//       through the receiver interpolation) in one launch of the step
//       kernel over both wavefields (k_a2<MODE, 2>, k_acoustic2d.cu), which
//       also accumulates the imaging condition below
//   compute_gradient! (src/fdtd/gradient.jl:27-56):
//       g_invK += p2_prev (p1_prev - p1) dtI                 (every p cell)
//       bx = vx2_prev (vx1 - vx1_prev) dtI, bz likewise      (velocity grids)
//       g_rho[iz+h, ix+h] -= (bx[iz+h, ix] + bx[iz+h, ix+1]) / 2
//                          + (bz[iz, ix+h] + bz[iz+1, ix+h]) / 2,
//       iz in 1..nz-2h, ix in 1..nx-2h (the averages sit four and five
//       cells off the velocity cells whose coefficients hold rho(r, c), as in
//       the reference); with Plan::d.imaging = 1 instead
//       g_rho[r, c] -= (bx[r, c+2] + bx[r, c+3]) / 2 + (bz[r+2, c] + bz[r+3, c]) / 2
//       over the updated velocity cells: the gradient of the discrete model
//       (dt / avg(rho) at vx cell c averages rho at c-3 and c-2)
// The time-reversal adjoint accumulates g_invK and, per velocity cell, the
// sums of bx and bz over the steps inside the step kernel; k_img_rho forms
// g_rho from those sums after the last step (the averages are linear, so
// only the summation order differs from the reference's per-step form).
// The checkpointed adjoint (gpi_ckpt.cu) runs the imaging condition as its
// own streaming pass over both wavefields' old and new states (k_grad_a2),
// with the velocity terms recomputed at the two neighbours each g_rho cell
// needs, in the reference's operation order.
#include "k_stencil.cuh"

namespace gpi {

struct GradArgs {
  int nz, nx, NZP;
  int64_t fs;
  int nshots;
  const float *p1A, *p1B, *p2A;
  const float *vx1A, *vx1B, *vx2A;
  const float *vz1A, *vz1B, *vz2A;
  const float *prev;  // strip values before boundary_force! (x strips, then z strips)
  int64_t pstride;    // floats per shot in prev
  int nb, npx, npz;   // strip width and PML offsets of the strips
  float *gK, *gR;
  float dtI;
  int imaging;  // 0 the reference's rho term, 1 the discrete model's
};

// position of p cell (r, c) in the strip block of boundary_save! (x strips
// nz x 2nb, then z strips 2nb x nx), -1 when the cell is in no strip
__device__ __forceinline__ int64_t strip_index(const GradArgs &a, int r, int c) {
  const int nb = a.nb;
  int j = -1;
  if (c > a.npx && c <= a.npx + nb)
    j = c - a.npx - 1;
  else if (c > a.nx - a.npx - nb && c <= a.nx - a.npx)
    j = nb + c - (a.nx - a.npx - nb) - 1;
  if (j >= 0) return (int64_t)(r - 1) + (int64_t)a.nz * j;
  if (r > a.npz && r <= a.npz + nb)
    j = r - a.npz - 1;
  else if (r > a.nz - a.npz - nb && r <= a.nz - a.npz)
    j = nb + r - (a.nz - a.npz - nb) - 1;
  if (j >= 0) return (int64_t)a.nz * 2 * nb + j + (int64_t)2 * nb * (c - 1);
  return -1;
}

__global__ void __launch_bounds__(256) k_grad_a2(const GradArgs a) {
  const int64_t per = (int64_t)a.nz * a.nx;
  const int64_t total = per * a.nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i - shot * per;
    const int r = (int)(k % a.nz) + 1, c = (int)(k / a.nz) + 1;
    const int64_t so = shot * a.fs;
    auto S = [&](int rr, int cc) -> int64_t { return so + (int64_t)(cc + XOFF - 1) * a.NZP + (rr + ZOFF - 1); };
    const int64_t o = S(r, c);
    // compute_gmodKI!
    float p1p = a.p1A[o];
    const int64_t sidx = strip_index(a, r, c);
    if (sidx >= 0) p1p = a.prev[shot * a.pstride + sidx];
    a.gK[o] = a.gK[o] + a.p2A[o] * (p1p - a.p1B[o]) * a.dtI;
    if (a.imaging) {
      // rho(r, c) sits in the coefficients of vx (r, c+2), (r, c+3) and vz
      // (r+2, c), (r+3, c) where those are updated (vx rows 4..nz-3,
      // columns 4..nx; vz rows 4..nz, columns 4..nx-3)
      auto bx = [&](int cc) {
        const int64_t q = S(r, cc);
        return cc >= 4 && cc <= a.nx ? a.vx2A[q] * (a.vx1B[q] - a.vx1A[q]) * a.dtI : 0.f;
      };
      auto bz = [&](int rr) {
        const int64_t q = S(rr, c);
        return rr >= 4 && rr <= a.nz ? a.vz2A[q] * (a.vz1B[q] - a.vz1A[q]) * a.dtI : 0.f;
      };
      const float avx = r >= 4 && r <= a.nz - 3 ? (bx(c + 2) + bx(c + 3)) * 0.5f : 0.f;
      const float avz = c >= 4 && c <= a.nx - 3 ? (bz(r + 2) + bz(r + 3)) * 0.5f : 0.f;
      a.gR[o] = a.gR[o] - avx - avz;
    } else if (r >= 4 && r <= a.nz - 3 && c >= 4 && c <= a.nx - 3) {
      // compute_gmodrho! + combine_gmodrho!
      const int64_t x1 = S(r, c - 3), x2 = S(r, c - 2), z1 = S(r - 3, c), z2 = S(r - 2, c);
      const float bx1 = a.vx2A[x1] * (a.vx1B[x1] - a.vx1A[x1]) * a.dtI;
      const float bx2 = a.vx2A[x2] * (a.vx1B[x2] - a.vx1A[x2]) * a.dtI;
      const float bz1 = a.vz2A[z1] * (a.vz1B[z1] - a.vz1A[z1]) * a.dtI;
      const float bz2 = a.vz2A[z2] * (a.vz1B[z2] - a.vz1A[z2]) * a.dtI;
      a.gR[o] = a.gR[o] - (bx1 + bx2) * 0.5f - (bz1 + bz2) * 0.5f;
    }
  }
}

// the imaging condition with wavefield 1's old (A) and new (B) states given
// explicitly and no strip values (the checkpointed adjoint)
int grad_a2_launch(Plan *p, const float *p1A, const float *p1B, const float *vx1A, const float *vx1B,
                   const float *vz1A, const float *vz1B) {
  GradArgs g;
  g.nz = p->d.nz;
  g.nx = p->d.nx;
  g.NZP = p->NZP;
  g.fs = p->fstride;
  g.nshots = p->d.nshots;
  g.p1A = p1A;
  g.p1B = p1B;
  const int A2 = p->cur[1];
  g.p2A = p->state[A2][1][GPI_P];
  g.vx1A = vx1A;
  g.vx1B = vx1B;
  g.vx2A = p->state[A2][1][GPI_VX];
  g.vz1A = vz1A;
  g.vz1B = vz1B;
  g.vz2A = p->state[A2][1][GPI_VZ];
  g.prev = nullptr;
  g.pstride = 0;
  g.nb = 0;  // no strip replaces a value
  g.npx = g.npz = 0;
  g.gK = p->grad[0];
  g.gR = p->grad[1];
  g.dtI = (float)(1.0 / p->d.dt);
  g.imaging = p->d.imaging;
  k_grad_a2<<<152 * 16, 256, 0, p->stream>>>(g);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

int step_adjoint_acoustic2d(Plan *p, int it) {
  (void)it;
  if (!p->grad[0] || !p->grad[1] || !p->bprev || !p->img[0] || !p->img[1])
    return fail(p, GPI_E_STATE, "adjoint step without gradient buffers");
  // wavefield 1 (time reversal, boundary already forced), wavefield 2 and
  // the imaging condition in one pass over the state
  return step_a2_adjoint_fused(p);
}

// The rho gradient from the per-velocity-cell sums hx, hz of the adjoint
// run (compute_gmodrho! + combine_gmodrho!, src/fdtd/gradient.jl:31-56, with
// the sum over the steps taken before the neighbour averages):
//   imaging 0: g_rho[r, c] = -(hx[r, c-3] + hx[r, c-2]) / 2 - (hz[r-3, c] + hz[r-2, c]) / 2,
//              r in 4..nz-3, c in 4..nx-3
//   imaging 1: g_rho[r, c] = -(hx[r, c+2] + hx[r, c+3]) / 2 - (hz[r+2, c] + hz[r+3, c]) / 2
//              over the updated velocity cells (vx rows 4..nz-3, columns
//              4..nx; vz rows 4..nz, columns 4..nx-3)
__global__ void __launch_bounds__(256) k_img_rho(const float *hx, const float *hz, float *gR, int nz, int nx, int NZP,
                                                 int64_t fs, int nshots, int imaging) {
  const int64_t per = (int64_t)nz * nx;
  const int64_t total = per * nshots;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int shot = (int)(i / per);
    const int64_t k = i - shot * per;
    const int r = (int)(k % nz) + 1, c = (int)(k / nz) + 1;
    const int64_t so = shot * fs;
    auto S = [&](int rr, int cc) -> int64_t { return so + (int64_t)(cc + XOFF - 1) * NZP + (rr + ZOFF - 1); };
    const int64_t o = S(r, c);
    if (imaging) {
      auto bx = [&](int cc) { return cc >= 4 && cc <= nx ? hx[S(r, cc)] : 0.f; };
      auto bz = [&](int rr) { return rr >= 4 && rr <= nz ? hz[S(rr, c)] : 0.f; };
      const float avx = r >= 4 && r <= nz - 3 ? (bx(c + 2) + bx(c + 3)) * 0.5f : 0.f;
      const float avz = c >= 4 && c <= nx - 3 ? (bz(r + 2) + bz(r + 3)) * 0.5f : 0.f;
      gR[o] = gR[o] - avx - avz;
    } else if (r >= 4 && r <= nz - 3 && c >= 4 && c <= nx - 3) {
      gR[o] = gR[o] - (hx[S(r, c - 3)] + hx[S(r, c - 2)]) * 0.5f - (hz[S(r - 3, c)] + hz[S(r - 2, c)]) * 0.5f;
    }
  }
}

int img_rho_finish(Plan *p) {
  k_img_rho<<<152 * 16, 256, 0, p->stream>>>(p->img[0], p->img[1], p->grad[1], p->d.nz, p->d.nx, p->NZP, p->fstride,
                                              p->d.nshots, p->d.imaging);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

}  // namespace gpi
