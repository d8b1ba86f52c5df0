// k_born.cu -- linearised (Born) modelling, 2-D acoustic.
//
// Wavefield 1 is the background run; wavefield 2 is its first-order
// perturbation for a medium perturbation (dinvK, drho).  Linearising one
// step of the scheme
//     v' = v + A (grad p)   (A = dt / avg(rho) at the velocity cell)
//     p' = p + B (div v')   (B = dt / invK at the p cell)
// gives the same scheme for the perturbation plus two secondary sources that
// need no derivatives: (dA / A) (v1' - v1) on the velocities and
// (dB / B) (p1' - p1) on p, with dA / A = -(drho_a + drho_b) / (rho_a +
// rho_b) over the two density cells of the velocity cell's coefficient (the
// same cells as the coefficient, src/fdtd/medium.jl:191-221, one cell off
// the stencil centre at order 4) and dB / B = -dinvK / invK.  Sources of
// wavefield 1 scale with the same A and B (src/fdtd/source.jl:61-157), so
// they are part of (v1' - v1) and (p1' - p1).  The reference's Born kernels
// (src/fdtd/born.jl:1-13) call compute_v!/compute_p! with arguments those
// kernels do not take; this is the operator they aim at, in the engine's
// own form.  A step: wavefield 1's fused step (A -> B), the velocity
// sources added to wavefield 2's input buffer, wavefield 2's fused step,
// the pressure sources added to its output buffer.
#include "gpi_internal.cuh"

namespace gpi {

int step_a2_wavefield(Plan *p, int ipw, int vonly);  // k_acoustic2d.cu

struct BornCoefArgs {
  int nz, nx, NZP;
  const float *invK, *rho, *dK, *dR;
  float *rp, *rvx, *rvz;
};

__global__ void k_born_coef(const BornCoefArgs a) {
  const int64_t n1 = a.nz + 3, total = n1 * (a.nx + 3);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i % n1) + 1, c = (int)(i / n1) + 1;
    auto S = [&](int rr, int cc) -> int64_t { return (int64_t)(cc + XOFF - 1) * a.NZP + (rr + ZOFF - 1); };
    const int64_t o = S(r, c);
    if (r <= a.nz && c <= a.nx) a.rp[o] = -(a.dK[o] / a.invK[o]);
    // vx cell (r, c): rho at (r, c-3), (r, c-2); updated rows 4..nz-3, columns 4..nx
    if (r >= 4 && r <= a.nz - 3 && c >= 4 && c <= a.nx) {
      const int64_t p0 = S(r, c - 3), p1 = S(r, c - 2);
      a.rvx[o] = -((a.dR[p0] + a.dR[p1]) / (a.rho[p0] + a.rho[p1]));
    }
    // vz cell (r, c): rho at (r-3, c), (r-2, c); updated rows 4..nz, columns 4..nx-3
    if (r >= 4 && r <= a.nz && c >= 4 && c <= a.nx - 3) {
      const int64_t p0 = S(r - 3, c), p1 = S(r - 2, c);
      a.rvz[o] = -((a.dR[p0] + a.dR[p1]) / (a.rho[p0] + a.rho[p1]));
    }
  }
}

// dst += r * (now - prev) over every shot; r holds one shot's cells
struct BornAddArgs {
  int64_t fs, total;
  int nf;
  float *dst[2];
  const float *r[2], *now[2], *prev[2];
};

__global__ void __launch_bounds__(256) k_born_add(const BornAddArgs a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i % a.fs;
    for (int f = 0; f < a.nf; f++) a.dst[f][i] = a.dst[f][i] + a.r[f][k] * (a.now[f][i] - a.prev[f][i]);
  }
}

int born_coefficients(Plan *p) {
  float *rp = p->born, *rvx = rp + p->fstride, *rvz = rvx + p->fstride;
  GPI_CUDA(p, cudaMemsetAsync(rp, 0, 3 * p->fstride * sizeof(float), p->stream));
  BornCoefArgs a;
  a.nz = p->d.nz;
  a.nx = p->d.nx;
  a.NZP = p->NZP;
  a.invK = p->mod[0];
  a.rho = p->mod[1];
  a.dK = rvz + p->fstride;
  a.dR = a.dK + p->fstride;
  a.rp = rp;
  a.rvx = rvx;
  a.rvz = rvz;
  k_born_coef<<<152 * 8, 256, 0, p->stream>>>(a);
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

static int born_add(Plan *p, int nf, float *const *dst, const float *const *r, const float *const *now,
                    const float *const *prev) {
  BornAddArgs a;
  a.fs = p->fstride;
  a.total = p->fstride * p->d.nshots;
  a.nf = nf;
  for (int f = 0; f < nf; f++) {
    a.dst[f] = dst[f];
    a.r[f] = r[f];
    a.now[f] = now[f];
    a.prev[f] = prev[f];
  }
  k_born_add<<<152 * 16, 256, 0, p->stream>>>(a);
  p->launches++;
  GPI_CUDA(p, cudaGetLastError());
  return GPI_OK;
}

// one Born step (after aux_step): see the file comment
static int born_step(Plan *p) {
  const float *rp = p->born, *rvx = rp + p->fstride, *rvz = rvx + p->fstride;
  int rc = step_a2_wavefield(p, 0, 0);
  if (rc) return rc;
  const int N1 = p->cur[0], O1 = N1 ^ 1, A2 = p->cur[1];
  {
    float *dst[2] = {p->state[A2][1][GPI_VX], p->state[A2][1][GPI_VZ]};
    const float *r[2] = {rvx, rvz};
    const float *now[2] = {p->state[N1][0][GPI_VX], p->state[N1][0][GPI_VZ]};
    const float *prev[2] = {p->state[O1][0][GPI_VX], p->state[O1][0][GPI_VZ]};
    if ((rc = born_add(p, 2, dst, r, now, prev))) return rc;
  }
  if ((rc = step_a2_wavefield(p, 1, 0))) return rc;
  float *dst[1] = {p->state[p->cur[1]][1][GPI_P]};
  const float *r[1] = {rp};
  const float *now[1] = {p->state[N1][0][GPI_P]};
  const float *prev[1] = {p->state[O1][0][GPI_P]};
  return born_add(p, 1, dst, r, now, prev);
}

int born_run(Plan *p) {
  p->rec_ipw = 1;
  int rc = GPI_OK;
  for (int it = 1; !rc && it <= p->d.nt; it++) {
    rc = aux_step(p, it, GPI_BORN);
    if (!rc) rc = born_step(p);
  }
  if (!rc) rc = aux_step(p, p->d.nt + 1, GPI_BORN);  // velocity records of the last step
  p->rec_ipw = 0;
  return rc;
}

}  // namespace gpi
