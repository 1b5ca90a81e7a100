// 2-D Diffusion and Allen-Cahn explicit steps with temporal blocking.
//
// One CTA owns a TY x TX output tile. It stages the tile plus a halo of
// `depth` cells (ghost rule applied at load time) in shared memory with
// 16-byte vector loads, advances `depth` time steps in shared memory (the
// valid region shrinks by one cell per step) and writes only the centre back:
// HBM sees one read and one write per cell per `depth` steps.
//
// Reference: engine_ExplicitDiffusion (Engines/Diffusion.py:198-208) and
// engine_CahnAllenExplicit (Engines/CahnAllen.py:128-135), with Field.laplacian
// (field.py:60-67) as the 5-point stencil.
#include "ppf_common.cuh"

namespace ppf {
namespace {

// c + dt*D*lap(c). The neighbour sum is grouped ((w+e)+(n+s)) so that a
// mirrored tile (no-flux ghosts deeper than one cell) evolves bit-identically
// to the cells it mirrors.
template <typename T>
struct DiffusionOp {
  T r;  // dt*D/dx^2
  __device__ __forceinline__ T operator()(T c, T w, T e, T n, T s) const {
    const T lap = ((w + e) + (n + s)) - T(4) * c;
    return c + r * lap;
  }
};

// phi + dt*M*(eps^2 lap(phi) - 16 W (4phi^3 - 6phi^2 + 2phi)).
template <typename T>
struct AllenCahnOp {
  T a;  // dt*M*eps^2/dx^2
  T b;  // dt*M*16*W
  __device__ __forceinline__ T operator()(T c, T w, T e, T n, T s) const {
    const T lap = ((w + e) + (n + s)) - T(4) * c;
    const T fp = c * (T(2) + c * (T(-6) + T(4) * c));
    return c + (a * lap - b * fp);
  }
};

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int n = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int n = 2;
};

constexpr int kThreads = 256;  // 8 warps; threadIdx.x = lane

// Shared-memory tile: H = TY + 2K rows of SW = TX + 2*KA columns, where
// KA = K rounded up to the 16-byte vector so that interior tiles load with
// aligned vector reads. Column KA - K is the first column used.
template <typename T, typename Op>
__global__ void __launch_bounds__(kThreads)
    stencil2d_tb_kernel(Op op, Geo g, Bc<T> bc, const T* __restrict__ in,
                        T* __restrict__ out, int TX, int TY, int K, int KA,
                        int vec_ok) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int V = Vec16<T>::n;
  using VT = typename Vec16<T>::type;
  const int SW = TX + 2 * KA;
  const int H = TY + 2 * K;
  T* buf0 = reinterpret_cast<T*>(smem_raw);
  T* buf1 = buf0 + (size_t)SW * H;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int ny = g.n[0], nx = g.n[1];

  pdl_wait();
  pdl_launch_next();

  const bool interior = vec_ok && (x0 - KA >= 0) && (y0 - K >= 0) &&
                        (x0 + TX + KA <= nx) && (y0 + TY + K <= ny);
  if (interior) {
    const int vpr = SW / V;  // vectors per smem row
    const int total = vpr * H;
    const T* src = in + (int64_t)(y0 - K) * g.pitch + (x0 - KA);
    constexpr int B = 4;
    for (int base = tid; base < total; base += kThreads * B) {
      VT r[B];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int i = base + u * kThreads;
        if (i < total) {
          const int ly = i / vpr, vx = i - ly * vpr;
          r[u] = __ldg(reinterpret_cast<const VT*>(src + (int64_t)ly * g.pitch) + vx);
        }
      }
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int i = base + u * kThreads;
        if (i < total) {
          const int ly = i / vpr, vx = i - ly * vpr;
          reinterpret_cast<VT*>(buf0 + (size_t)ly * SW)[vx] = r[u];
        }
      }
    }
  } else {
    for (int ly = threadIdx.y; ly < H; ly += kThreads / 32) {
      const int gy = y0 - K + ly;
      for (int lx = KA - K + threadIdx.x; lx < KA + TX + K; lx += 32) {
        const int gx = x0 - KA + lx;
        buf0[ly * SW + lx] = fetch<T, 2>(in, g, bc, 0, gy, gx);
      }
    }
  }
  __syncthreads();

  // Sub-steps 1..K-1 stay in shared memory; step K writes the centre tile.
  T* src = buf0;
  T* dst = buf1;
  for (int s = 1; s < K; ++s) {
    for (int ly = s + threadIdx.y; ly < H - s; ly += kThreads / 32) {
      const int gy = y0 - K + ly;
      const T* row = src + ly * SW;
      T* orow = dst + ly * SW;
      for (int lx = KA - K + s + threadIdx.x; lx < KA + TX + K - s; lx += 32) {
        const T c = row[lx];
        T v;
        if (!interior && dirichlet_ghost<T, 2>(g, bc, gy, x0 - KA + lx))
          v = c;
        else
          v = op(c, row[lx - 1], row[lx + 1], row[lx - SW], row[lx + SW]);
        orow[lx] = v;
      }
    }
    __syncthreads();
    T* t = src;
    src = dst;
    dst = t;
  }
  for (int ly = K + threadIdx.y; ly < K + TY; ly += kThreads / 32) {
    const int gy = y0 - K + ly;
    if (gy >= ny) break;
    const T* row = src + ly * SW;
    T* orow = out + (int64_t)gy * g.pitch;
    for (int lx = KA + threadIdx.x; lx < KA + TX; lx += 32) {
      const int gx = x0 - KA + lx;
      if (gx >= nx) break;
      const T c = row[lx];
      orow[gx] = op(c, row[lx - 1], row[lx + 1], row[lx - SW], row[lx + SW]);
    }
  }
}

// Lean depth-1 kernel: a warp owns WW = 32 V columns (V cells of one
// 16-byte vector per lane) and kRB rows. It requests the kRB + 2 rows it
// reads (band plus halo rows) as vector loads up front, takes the west /
// east neighbours across lanes by shuffles (lanes 0 and 31 load the strip's
// outer neighbours), and writes each output row as one vector per lane: no
// shared memory, no barriers. Edge bands use the generic ghost rule.
constexpr int kRB = 8;

template <typename T, typename Op>
__global__ void __launch_bounds__(kThreads)
    stencil2d_lean_kernel(Op op, Geo g, Bc<T> bc, const T* __restrict__ in, T* __restrict__ out,
                          int vec_ok) {
  constexpr int V = Vec16<T>::n;
  using VT = typename Vec16<T>::type;
  constexpr int WW = 32 * V;
  const int lane = threadIdx.x;
  const int x0 = blockIdx.x * WW;
  const int y0 = (blockIdx.y * (kThreads / 32) + threadIdx.y) * kRB;
  const int ny = g.n[0], nx = g.n[1];
  pdl_wait();
  pdl_launch_next();
  if (y0 >= ny) return;  // whole warp
  // full strips whose rows y0 - 1 .. y0 + kRB lie inside the grid take the
  // vector path; the left / right edge strips fetch their one ghost column
  // through the boundary rule (lanes 0 / 31 only)
  const bool fast = vec_ok && x0 + WW <= nx && y0 >= 1 && y0 + kRB + 1 <= ny;
  if (fast) {
    const T* base = in + (int64_t)(y0 - 1) * g.pitch + x0;
    VT r[kRB + 2];
#pragma unroll
    for (int j = 0; j < kRB + 2; ++j)
      r[j] = __ldg(reinterpret_cast<const VT*>(base + (int64_t)j * g.pitch) + lane);
    T wv[kRB], ev[kRB];
#pragma unroll
    for (int j = 0; j < kRB; ++j) {
      const T* row = base + (int64_t)(j + 1) * g.pitch;
      if (lane == 0)
        wv[j] = x0 >= 1 ? __ldg(row - 1) : fetch<T, 2>(in, g, bc, 0, y0 + j, x0 - 1);
      else
        wv[j] = T(0);
      if (lane == 31)
        ev[j] = x0 + WW + 1 <= nx ? __ldg(row + WW) : fetch<T, 2>(in, g, bc, 0, y0 + j, x0 + WW);
      else
        ev[j] = T(0);
    }
    T* obase = out + (int64_t)y0 * g.pitch + x0 + lane * V;
#pragma unroll
    for (int j = 1; j <= kRB; ++j) {
      const T* c = reinterpret_cast<const T*>(&r[j]);
      const T* n = reinterpret_cast<const T*>(&r[j - 1]);
      const T* sv = reinterpret_cast<const T*>(&r[j + 1]);
      T wl = __shfl_up_sync(0xffffffffu, c[V - 1], 1);
      T er = __shfl_down_sync(0xffffffffu, c[0], 1);
      if (lane == 0) wl = wv[j - 1];
      if (lane == 31) er = ev[j - 1];
      VT o;
      T* ov = reinterpret_cast<T*>(&o);
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const T w = e == 0 ? wl : c[e - 1];
        const T ea = e == V - 1 ? er : c[e + 1];
        ov[e] = op(c[e], w, ea, n[e], sv[e]);
      }
      *reinterpret_cast<VT*>(obase + (int64_t)(j - 1) * g.pitch) = o;
    }
  } else {
    for (int j = 0; j < kRB; ++j) {
      const int row = y0 + j;
      if (row >= ny) break;
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const int x = x0 + lane * V + e;
        if (x < nx)
          out[(int64_t)row * g.pitch + x] =
              op(fetch<T, 2>(in, g, bc, 0, row, x), fetch<T, 2>(in, g, bc, 0, row, x - 1),
                 fetch<T, 2>(in, g, bc, 0, row, x + 1), fetch<T, 2>(in, g, bc, 0, row - 1, x),
                 fetch<T, 2>(in, g, bc, 0, row + 1, x));
      }
    }
  }
}

struct Tile2d {
  int tx, ty, k, ka;
  size_t smem;
};

template <typename T>
int32_t plan_tile2d(const PpfTiling* t, Tile2d* out) {
  Tile2d r;
  r.k = t && t->depth ? t->depth : 1;
  r.tx = t && t->tile_x ? t->tile_x : (sizeof(T) == 4 ? 128 : 64);
  r.ty = t && t->tile_y ? t->tile_y : 32;
  if (r.k < 1 || r.k > 8)
    return fail(PPF_ERR_INVALID, "depth=%d not in [1, 8]", r.k);
  if (r.tx < 8 || r.tx > 1024 || (r.tx % 4) != 0 || r.ty < 1 || r.ty > 1024)
    return fail(PPF_ERR_INVALID, "tile %dx%d invalid (tile_x multiple of 4)",
                r.tx, r.ty);
  const int V = 16 / (int)sizeof(T);
  r.ka = (r.k + V - 1) / V * V;
  const size_t one = (size_t)(r.tx + 2 * r.ka) * (r.ty + 2 * r.k) * sizeof(T);
  r.smem = r.k > 1 ? 2 * one : one;
  if (r.smem > 200 * 1024)
    return fail(PPF_ERR_INVALID, "tile needs %zu bytes of shared memory",
                r.smem);
  *out = r;
  return PPF_OK;
}

template <typename T, typename Op>
int32_t run2d(Op op, double dx, const PpfGrid* grid, const PpfBoundary* b,
              const T* in, T* out, const PpfTiling* tiling, void* stream) {
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (in == out) return fail(PPF_ERR_INVALID, "in and out must differ");
  Tile2d t;
  if ((rc = plan_tile2d<T>(tiling, &t))) return rc;
  Bc<T> bc;
  if ((rc = make_bc<T>(b, g, dx, 1, t.k, &bc))) return rc;
  const int vec_ok = (((uintptr_t)in) % 16 == 0) && (((uintptr_t)out) % 16 == 0) &&
                     ((g.pitch * sizeof(T)) % 16 == 0);
  const bool pdl = tiling && tiling->pdl;
  if (t.k == 1 && !(tiling && (tiling->tile_x || tiling->tile_y))) {
    constexpr int WW = 32 * Vec16<T>::n;
    dim3 grid_dim((g.n[1] + WW - 1) / WW,
                  (g.n[0] + kRB * (kThreads / 32) - 1) / (kRB * (kThreads / 32)));
    if (grid_dim.y > 65535) return fail(PPF_ERR_INVALID, "too many row bands");
    PPF_TRY_CUDA(launch(stencil2d_lean_kernel<T, Op>, grid_dim, dim3(32, kThreads / 32), 0,
                        (cudaStream_t)stream, pdl, op, g, bc, in, out, vec_ok));
    return PPF_OK;
  }
  auto kern = stencil2d_tb_kernel<T, Op>;
  PPF_TRY_CUDA(allow_smem(kern, t.smem));
  dim3 grid_dim((g.n[1] + t.tx - 1) / t.tx, (g.n[0] + t.ty - 1) / t.ty);
  if (grid_dim.y > 65535) return fail(PPF_ERR_INVALID, "too many tile rows");
  PPF_TRY_CUDA(launch(kern, grid_dim, dim3(32, kThreads / 32), t.smem,
                      (cudaStream_t)stream, pdl, op, g, bc, in, out, t.tx,
                      t.ty, t.k, t.ka, vec_ok));
  return PPF_OK;
}

template <typename T>
int32_t diffusion(const PpfDiffusionParams* p, const PpfGrid* g,
                  const PpfBoundary* b, const T* in, T* out,
                  const PpfTiling* t, void* s) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  if (!(p->dx > 0)) return fail(PPF_ERR_INVALID, "dx must be > 0");
  DiffusionOp<T> op{(T)(p->dt * p->D / (p->dx * p->dx))};
  return run2d<T>(op, p->dx, g, b, in, out, t, s);
}

template <typename T>
int32_t allen_cahn(const PpfAllenCahnParams* p, const PpfGrid* g,
                   const PpfBoundary* b, const T* in, T* out,
                   const PpfTiling* t, void* s) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  if (!(p->dx > 0)) return fail(PPF_ERR_INVALID, "dx must be > 0");
  AllenCahnOp<T> op{(T)(p->dt * p->M * p->epsilon * p->epsilon / (p->dx * p->dx)),
                    (T)(p->dt * p->M * 16.0 * p->W)};
  return run2d<T>(op, p->dx, g, b, in, out, t, s);
}

}  // namespace

// 3-D variants live in stencil3d.cu.
int32_t diffusion3d_f32(const PpfDiffusionParams*, const PpfGrid*,
                        const PpfBoundary*, const float*, float*,
                        const PpfTiling*, void*);
int32_t diffusion3d_f64(const PpfDiffusionParams*, const PpfGrid*,
                        const PpfBoundary*, const double*, double*,
                        const PpfTiling*, void*);
int32_t allen_cahn3d_f32(const PpfAllenCahnParams*, const PpfGrid*,
                         const PpfBoundary*, const float*, float*,
                         const PpfTiling*, void*);
int32_t allen_cahn3d_f64(const PpfAllenCahnParams*, const PpfGrid*,
                         const PpfBoundary*, const double*, double*,
                         const PpfTiling*, void*);

}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_diffusion_step_f32(const PpfDiffusionParams* p, const PpfGrid* g,
                               const PpfBoundary* bc, const float* in,
                               float* out, const PpfTiling* tiling,
                               void* stream) {
  if (g && g->ndim == 3) return diffusion3d_f32(p, g, bc, in, out, tiling, stream);
  return diffusion<float>(p, g, bc, in, out, tiling, stream);
}
int32_t ppf_diffusion_step_f64(const PpfDiffusionParams* p, const PpfGrid* g,
                               const PpfBoundary* bc, const double* in,
                               double* out, const PpfTiling* tiling,
                               void* stream) {
  if (g && g->ndim == 3) return diffusion3d_f64(p, g, bc, in, out, tiling, stream);
  return diffusion<double>(p, g, bc, in, out, tiling, stream);
}
int32_t ppf_allen_cahn_step_f32(const PpfAllenCahnParams* p, const PpfGrid* g,
                                const PpfBoundary* bc, const float* in,
                                float* out, const PpfTiling* tiling,
                                void* stream) {
  if (g && g->ndim == 3) return allen_cahn3d_f32(p, g, bc, in, out, tiling, stream);
  return allen_cahn<float>(p, g, bc, in, out, tiling, stream);
}
int32_t ppf_allen_cahn_step_f64(const PpfAllenCahnParams* p, const PpfGrid* g,
                                const PpfBoundary* bc, const double* in,
                                double* out, const PpfTiling* tiling,
                                void* stream) {
  if (g && g->ndim == 3) return allen_cahn3d_f64(p, g, bc, in, out, tiling, stream);
  return allen_cahn<double>(p, g, bc, in, out, tiling, stream);
}

}  // extern "C"
