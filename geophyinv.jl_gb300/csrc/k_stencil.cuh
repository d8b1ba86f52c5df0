// k_stencil.cuh -- device helpers shared by the fused step kernels.
#pragma once
#include "gpi_internal.cuh"

namespace gpi {

// 4th-order staggered difference 27 a2 - 27 a1 + a0 - a3
// (@d_?a / @d_?i at order 4, src/fdtd/diff2D.jl:62-97)
__device__ __forceinline__ float st4(float a0, float a1, float a2, float a3) {
  return a2 * 27.0f - a1 * 27.0f + a0 - a3;
}

// CPML strip slot of derivative index i (1-based) on an axis of length nd,
// -1 outside the strips (memory{x,y,z}!, src/fdtd/cpml.jl:184-211)
__device__ __forceinline__ int pml_slot(int i, int nd, int npml, bool lo, bool hi) {
  if (lo && i <= npml) return i - 1;
  if (hi && i > nd - npml) return npml + i - (nd - npml) - 1;
  return -1;
}

// psi = b psi + a d ; d = d kI + psi   (src/fdtd/cpml.jl:175-182)
// pm points at this derivative's [a | b | kI] blocks of 2*npml each.
__device__ __forceinline__ float cpml(float D, const float *pm, int npml, int j, const float *psA, float *psB,
                                      int64_t po, bool own) {
  const float psi = pm[2 * npml + j] * psA[po] + pm[j] * D;
  if (own) psB[po] = psi;
  return D * pm[4 * npml + j] + psi;
}

// binary search of the first injection cell with column >= col in [lo, hi)
__device__ __forceinline__ int first_col(const InjCell *cells, int lo, int hi, int col) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cells[mid].col < col)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Per-kind cursor over injection cells sorted by column: every thread of a
// block walks the same cells column by column.
struct InjCursor {
  int cur, end, ncol;
  __device__ __forceinline__ void init(const InjCell *cells, int b, int e) {
    cur = b;
    end = e;
    ncol = cur < end ? cells[cur].col : 0x7fffffff;
  }
  // returns the [b, e) range of cells in column `col` and advances past it
  __device__ __forceinline__ void range(const InjCell *cells, int col, int &b, int &e) {
    b = cur;
    if (ncol == col) {
      while (cur < end && cells[cur].col == col) cur++;
      ncol = cur < end ? cells[cur].col : 0x7fffffff;
    }
    e = cur;
  }
};

__device__ __forceinline__ void inject(const InjCell *cells, const float *amount, int b, int e, int row, float &v) {
  for (int k = b; k < e; k++)
    if (cells[k].row == row) v = v + amount[k];
}

// Injection cells read through a view: column, row and amount of cell k at
// col[k * st], row[k * st], amt[k] -- the cells in global memory (st =
// sizeof(InjCell) / 4) or a block's copy in shared memory (st = 1).
struct InjView {
  const int *col, *row;
  const float *amt;
  int st;
};
struct InjVCursor {
  int cur, end, ncol;
  __device__ __forceinline__ void init(const InjView &v, int b, int e) {
    cur = b;
    end = e;
    ncol = cur < end ? v.col[cur * v.st] : 0x7fffffff;
  }
  // the [b, e) range of cells in column `col`, advancing past it
  __device__ __forceinline__ void range(const InjView &v, int col, int &b, int &e) {
    b = cur;
    if (ncol == col) {
      while (cur < end && v.col[cur * v.st] == col) cur++;
      ncol = cur < end ? v.col[cur * v.st] : 0x7fffffff;
    }
    e = cur;
  }
};
__device__ __forceinline__ void inject(const InjView &v, int b, int e, int row, float &x) {
  for (int k = b; k < e; k++)
    if (v.row[k * v.st] == row) x = x + v.amt[k];
}

// ---------------------------------------------------------------------------
// bulk asynchronous copies (TMA engine, 1-D form) completing on mbarriers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: gives up after `limit` polls and reports it
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int limit = 1 << 22) {
  for (int i = 0; i < limit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace gpi
