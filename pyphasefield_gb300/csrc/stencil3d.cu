// 3-D explicit steps that march along z: Diffusion / Allen-Cahn (7-point)
// and Cahn-Hilliard (radius 2 through an on-chip chemical-potential tile).
//
// A CTA owns a TY x TX column of the grid and a chunk of ZC planes. It keeps
// a ring of z-planes (with an xy halo) in shared memory, loads each plane
// once, and writes each updated plane once, so HBM sees one read and one
// write per cell per step; xy halos are re-read from L2.
//
// Reference: Field.laplacian (field.py:60-67), engine_ExplicitDiffusion
// (Engines/Diffusion.py:198-208), engine_CahnAllenExplicit
// (Engines/CahnAllen.py:128-135), engine_CahnHilliardExplicit
// (Engines/CahnHilliard.py:134-146).
#include <cmath>

#include "ppf_common.cuh"

namespace ppf {
namespace {

constexpr int kThreads = 256;

template <typename T>
struct Diffusion7 {
  T r;
  __device__ __forceinline__ T operator()(T c, T w, T e, T n, T s, T d,
                                          T u) const {
    const T lap = (((w + e) + (n + s)) + (d + u)) - T(6) * c;
    return c + r * lap;
  }
};

template <typename T>
struct AllenCahn7 {
  T a, b;
  __device__ __forceinline__ T operator()(T c, T w, T e, T n, T s, T d,
                                          T u) const {
    const T lap = (((w + e) + (n + s)) + (d + u)) - T(6) * c;
    const T fp = c * (T(2) + c * (T(-6) + T(4) * c));
    return c + (a * lap - b * fp);
  }
};

// Loads plane gz of `in` with an xy halo of `h` cells into `dst`
// ((TY+2h) x (TX+2h), row stride TX+2h). Interior tiles read directly.
template <typename T>
__device__ __forceinline__ void load_plane(T* dst, const T* __restrict__ in,
                                           const Geo& g, const Bc<T>& bc,
                                           int gz, int y0, int x0, int TX,
                                           int TY, int h, bool xy_interior) {
  const int W = TX + 2 * h, H = TY + 2 * h;
  const bool inside = xy_interior && (unsigned)gz < (unsigned)g.n[0];
  for (int ly = threadIdx.y; ly < H; ly += kThreads / 32) {
    const int gy = y0 - h + ly;
    if (inside) {
      const T* row = in + (int64_t)gz * g.plane + (int64_t)gy * g.pitch + (x0 - h);
      for (int lx = threadIdx.x; lx < W; lx += 32) dst[ly * W + lx] = __ldg(row + lx);
    } else {
      for (int lx = threadIdx.x; lx < W; lx += 32)
        dst[ly * W + lx] = fetch<T, 3>(in, g, bc, 0, gz, gy, x0 - h + lx);
    }
  }
}

// ------------------------------------------------------------- 7-point
template <typename T, typename Op>
__global__ void __launch_bounds__(kThreads)
    march7_kernel(Op op, Geo g, Bc<T> bc, const T* __restrict__ in,
                  T* __restrict__ out, int TX, int TY, int ZC) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int W = TX + 2, H = TY + 2, P = W * H;
  T* ring = reinterpret_cast<T*>(smem_raw);  // 3 planes
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * ZC;
  const int nz = g.n[0], ny = g.n[1], nx = g.n[2];
  const int z1 = min(z0 + ZC, nz);
  const bool xy_in = x0 >= 1 && y0 >= 1 && x0 + TX + 1 <= nx && y0 + TY + 1 <= ny;

  pdl_wait();
  pdl_launch_next();

  load_plane(ring + ((z0 - 1 + 3) % 3) * P, in, g, bc, z0 - 1, y0, x0, TX, TY, 1, xy_in);
  load_plane(ring + (z0 % 3) * P, in, g, bc, z0, y0, x0, TX, TY, 1, xy_in);
  for (int z = z0; z < z1; ++z) {
    load_plane(ring + ((z + 1) % 3) * P, in, g, bc, z + 1, y0, x0, TX, TY, 1, xy_in);
    __syncthreads();
    const T* pd = ring + ((z + 2) % 3) * P;  // z-1
    const T* pc = ring + (z % 3) * P;
    const T* pu = ring + ((z + 1) % 3) * P;
    for (int ly = 1 + threadIdx.y; ly <= TY; ly += kThreads / 32) {
      const int gy = y0 + ly - 1;
      if (gy >= ny) break;
      T* orow = out + (int64_t)z * g.plane + (int64_t)gy * g.pitch;
      for (int lx = 1 + threadIdx.x; lx <= TX; lx += 32) {
        const int gx = x0 + lx - 1;
        if (gx >= nx) break;
        const int i = ly * W + lx;
        orow[gx] = op(pc[i], pc[i - 1], pc[i + 1], pc[i - W], pc[i + W], pd[i], pu[i]);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- Cahn-Hilliard
// mu~ = -(eps^2/dx^2) lap'(c) + (4c^3 - 6c^2 + 2c), lap' the unscaled 7-point
// sum; c' = c + sum over the 6 faces of F = a (mu~_nbr - mu~_c), a = dt M/dx^2.
// With QUANT each face flux is rounded to a multiple of q (a power of two).
// F(A->B) = -F(B->A) bit for bit (the same mu~ values enter both cells and
// rounding to nearest is odd-symmetric), so the float field conserves its
// sum exactly while every value stays a multiple of q below 2^24 q.
template <typename T>
struct ChCoef {
  T kap;         // eps^2/dx^2
  T a;           // dt*M/dx^2
  T q, iq;       // quantum and its inverse (QUANT only)
  T range;       // 2^24 q: |c| beyond this loses exactness (QUANT only)
  int centered;  // field holds u = c - 1/2
};

template <typename T>
__device__ __forceinline__ T ch_mu(const ChCoef<T>& k, T c, T w, T e, T n,
                                   T s, T d, T u) {
  const T lap = (((w + e) + (n + s)) + (d + u)) - T(6) * c;
  // 4c^3 - 6c^2 + 2c, or in the centered variable 4u^3 - u
  const T fp = k.centered ? c * (T(4) * c * c - T(1))
                          : c * (T(2) + c * (T(-6) + T(4) * c));
  return fp - k.kap * lap;
}

template <typename T, bool QUANT>
__device__ __forceinline__ T ch_flux(const ChCoef<T>& k, T mn, T mc) {
  const T f = k.a * (mn - mc);
  if (QUANT) return rint(f * k.iq) * k.q;
  return f;
}

template <typename T, bool QUANT>
__global__ void __launch_bounds__(kThreads)
    cahn_hilliard_kernel(ChCoef<T> k, Geo g, Bc<T> bc, const T* __restrict__ in,
                         T* __restrict__ out, double* __restrict__ mass,
                         int* __restrict__ status, int TX, int TY, int ZC) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int WC = TX + 4, HC = TY + 4, PC = WC * HC;  // c planes, halo 2
  const int WM = TX + 2, HM = TY + 2, PM = WM * HM;  // mu planes, halo 1
  T* cring = reinterpret_cast<T*>(smem_raw);          // 5 planes
  T* mring = cring + 5 * PC;                          // 3 planes
  __shared__ double red[kThreads / 32];
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * ZC;
  const int nz = g.n[0], ny = g.n[1], nx = g.n[2];
  const int z1 = min(z0 + ZC, nz);
  const bool xy_in = x0 >= 2 && y0 >= 2 && x0 + TX + 2 <= nx && y0 + TY + 2 <= ny;

  pdl_wait();
  pdl_launch_next();

  auto cslot = [&](int z) { return cring + ((z % 5 + 5) % 5) * PC; };
  auto mslot = [&](int z) { return mring + ((z % 3 + 3) % 3) * PM; };
  // mu~ on the (TY+2) x (TX+2) region of plane z from c planes z-1, z, z+1.
  auto compute_mu = [&](int z) {
    const T* cd = cslot(z - 1);
    const T* cc = cslot(z);
    const T* cu = cslot(z + 1);
    T* m = mslot(z);
    for (int ly = threadIdx.y; ly < HM; ly += kThreads / 32)
      for (int lx = threadIdx.x; lx < WM; lx += 32) {
        const int i = (ly + 1) * WC + (lx + 1);
        m[ly * WM + lx] = ch_mu(k, cc[i], cc[i - 1], cc[i + 1], cc[i - WC],
                                cc[i + WC], cd[i], cu[i]);
      }
  };

  for (int z = z0 - 2; z <= z0 + 1; ++z)
    load_plane(cslot(z), in, g, bc, z, y0, x0, TX, TY, 2, xy_in);
  __syncthreads();
  compute_mu(z0 - 1);
  compute_mu(z0);

  double acc = 0.0;
  int flags = 0;
  for (int z = z0; z < z1; ++z) {
    load_plane(cslot(z + 2), in, g, bc, z + 2, y0, x0, TX, TY, 2, xy_in);
    __syncthreads();
    compute_mu(z + 1);
    __syncthreads();
    const T* md = mslot(z - 1);
    const T* mc = mslot(z);
    const T* mu = mslot(z + 1);
    const T* cc = cslot(z);
    for (int ly = 1 + threadIdx.y; ly <= TY; ly += kThreads / 32) {
      const int gy = y0 + ly - 1;
      if (gy >= ny) break;
      T* orow = out + (int64_t)z * g.plane + (int64_t)gy * g.pitch;
      for (int lx = 1 + threadIdx.x; lx <= TX; lx += 32) {
        const int gx = x0 + lx - 1;
        if (gx >= nx) break;
        const int i = ly * WM + lx;
        const T m0 = mc[i];
        const T fw = ch_flux<T, QUANT>(k, mc[i - 1], m0);
        const T fe = ch_flux<T, QUANT>(k, mc[i + 1], m0);
        const T fn = ch_flux<T, QUANT>(k, mc[i - WM], m0);
        const T fs = ch_flux<T, QUANT>(k, mc[i + WM], m0);
        const T fd = ch_flux<T, QUANT>(k, md[i], m0);
        const T fu = ch_flux<T, QUANT>(k, mu[i], m0);
        const T c0 = cc[(ly + 1) * WC + (lx + 1)];
        const T v = c0 + (((fw + fe) + (fn + fs)) + (fd + fu));
        orow[gx] = v;
        acc += (double)v;
        if (!isfinite(v)) flags |= PPF_STATUS_NONFINITE;
        if (QUANT && fabs(v) >= k.range) flags |= PPF_STATUS_RANGE;
      }
    }
  }
  if (status && flags) atomicOr(status, flags);
  if (mass) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    const int warp = threadIdx.y;
    if (threadIdx.x == 0) red[warp] = acc;
    __syncthreads();
    if (warp == 0) {
      double v = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) atomicAdd(mass, v);
    }
  }
}

struct Tile3d {
  int tx, ty, zc;
};

template <typename T>
int32_t plan3d(const PpfTiling* t, const Geo& g, int halo, int nplanes_c,
               int nplanes_m, Tile3d* r, size_t* smem) {
  r->tx = t && t->tile_x ? t->tile_x : 64;
  r->ty = t && t->tile_y ? t->tile_y : 16;
  if (t && t->depth > 1)
    return fail(PPF_ERR_UNSUPPORTED, "3-D steps advance one step per pass (depth=%d)",
                t->depth);
  if (r->tx < 1 || r->tx > 512 || r->ty < 1 || r->ty > 512)
    return fail(PPF_ERR_INVALID, "tile %dx%d invalid", r->tx, r->ty);
  // z chunk: enough CTAs for ~4 waves of 152 SMs, at least 8 planes.
  const long tiles = (long)((g.n[2] + r->tx - 1) / r->tx) * ((g.n[1] + r->ty - 1) / r->ty);
  int zc = (int)((long)g.n[0] * tiles / (152L * 4 * 2));
  zc = zc < 8 ? 8 : zc;
  zc = zc > 64 ? 64 : zc;
  r->zc = zc > g.n[0] ? g.n[0] : zc;
  *smem = ((size_t)nplanes_c * (r->tx + 2 * halo) * (r->ty + 2 * halo) +
           (size_t)nplanes_m * (r->tx + 2) * (r->ty + 2)) *
          sizeof(T);
  if (*smem > 200 * 1024)
    return fail(PPF_ERR_INVALID, "tile needs %zu bytes of shared memory", *smem);
  return PPF_OK;
}

// A 2-D grid runs as a single-plane 3-D grid with a periodic z axis (the
// z neighbours are the cell itself and cancel in the Laplacian).
int32_t as3d(const PpfGrid* in, const PpfBoundary* bin, PpfGrid* g3,
             PpfBoundary* b3) {
  if (!in) return fail(PPF_ERR_INVALID, "grid is NULL");
  if (!bin) return fail(PPF_ERR_INVALID, "boundary is NULL");
  *g3 = *in;
  *b3 = *bin;
  if (in->ndim == 2) {
    g3->ndim = 3;
    g3->shape[2] = in->shape[1];
    g3->shape[1] = in->shape[0];
    g3->shape[0] = 1;
    b3->type[2] = bin->type[1];
    b3->type[1] = bin->type[0];
    b3->type[0] = PPF_BC_PERIODIC;
    for (int f = 0; f < 2; ++f)
      for (int s = 0; s < 2; ++s) {
        b3->value[f][2][s] = bin->value[f][1][s];
        b3->value[f][1][s] = bin->value[f][0][s];
        b3->value[f][0][s] = 0.0;
      }
  }
  return PPF_OK;
}

template <typename T, typename Op>
int32_t run_march7(Op op, double dx, const PpfGrid* grid, const PpfBoundary* b,
                   const T* in, T* out, const PpfTiling* tiling, void* stream) {
  Geo g;
  int32_t rc = make_geo(grid, 3, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (in == out) return fail(PPF_ERR_INVALID, "in and out must differ");
  Bc<T> bc;
  if ((rc = make_bc<T>(b, g, dx, 1, 1, &bc))) return rc;
  Tile3d t;
  size_t smem;
  if ((rc = plan3d<T>(tiling, g, 1, 3, 0, &t, &smem))) return rc;
  auto kern = march7_kernel<T, Op>;
  PPF_TRY_CUDA(allow_smem(kern, smem));
  dim3 gd((g.n[2] + t.tx - 1) / t.tx, (g.n[1] + t.ty - 1) / t.ty,
          (g.n[0] + t.zc - 1) / t.zc);
  PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream,
                      tiling && tiling->pdl, op, g, bc, in, out, t.tx, t.ty, t.zc));
  return PPF_OK;
}

template <typename T>
int32_t cahn_hilliard(const PpfCahnHilliardParams* p, const PpfGrid* grid_in,
                      const PpfBoundary* b_in, const T* in, T* out,
                      double* mass, int32_t* status, const PpfTiling* tiling,
                      void* stream) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  if (!(p->dx > 0)) return fail(PPF_ERR_INVALID, "dx must be > 0");
  PpfGrid grid;
  PpfBoundary b;
  int32_t rc = as3d(grid_in, b_in, &grid, &b);
  if (rc) return rc;
  Geo g;
  if ((rc = make_geo(&grid, 3, 3, &g))) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (in == out) return fail(PPF_ERR_INVALID, "in and out must differ");
  for (int a = 0; a < 3; ++a) {
    if (b.type[a] == PPF_BC_DIRCHLET)
      return fail(PPF_ERR_UNSUPPORTED,
                  "Cahn-Hilliard supports PERIODIC and NEUMANN axes only");
    if (b.type[a] == PPF_BC_NEUMANN && (b.value[0][a][0] != 0.0 || b.value[0][a][1] != 0.0))
      return fail(PPF_ERR_UNSUPPORTED,
                  "Cahn-Hilliard NEUMANN axes must be no-flux (gradient 0)");
  }
  Bc<T> bc;
  if ((rc = make_bc<T>(&b, g, p->dx, 1, 2, &bc))) return rc;
  Tile3d t;
  size_t smem;
  if ((rc = plan3d<T>(tiling, g, 2, 5, 3, &t, &smem))) return rc;
  ChCoef<T> k;
  k.kap = (T)(p->epsilon * p->epsilon / (p->dx * p->dx));
  k.a = (T)(p->dt * p->M / (p->dx * p->dx));
  const bool quant = p->quantum > 0;
  if (quant) {
    int e;
    const double m = std::frexp(p->quantum, &e);
    if (m != 0.5 || sizeof(T) != 4)
      return fail(PPF_ERR_INVALID,
                  "quantum must be a power of two and needs the float path");
  }
  k.q = (T)(quant ? p->quantum : 0.0);
  k.iq = (T)(quant ? 1.0 / p->quantum : 0.0);
  k.range = (T)(quant ? std::ldexp(p->quantum, 24) : 0.0);
  if (p->centered != 0 && p->centered != 1)
    return fail(PPF_ERR_INVALID, "centered must be 0 or 1");
  k.centered = p->centered;
  dim3 gd((g.n[2] + t.tx - 1) / t.tx, (g.n[1] + t.ty - 1) / t.ty,
          (g.n[0] + t.zc - 1) / t.zc);
  const bool pdl = tiling && tiling->pdl;
  if (quant) {
    auto kern = cahn_hilliard_kernel<T, true>;
    PPF_TRY_CUDA(allow_smem(kern, smem));
    PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream,
                        pdl, k, g, bc, in, out, mass, (int*)status, t.tx, t.ty, t.zc));
  } else {
    auto kern = cahn_hilliard_kernel<T, false>;
    PPF_TRY_CUDA(allow_smem(kern, smem));
    PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream,
                        pdl, k, g, bc, in, out, mass, (int*)status, t.tx, t.ty, t.zc));
  }
  return PPF_OK;
}

}  // namespace

int32_t diffusion3d_f32(const PpfDiffusionParams* p, const PpfGrid* g,
                        const PpfBoundary* b, const float* in, float* out,
                        const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  return run_march7<float>(Diffusion7<float>{(float)(p->dt * p->D / (p->dx * p->dx))},
                           p->dx, g, b, in, out, t, s);
}
int32_t diffusion3d_f64(const PpfDiffusionParams* p, const PpfGrid* g,
                        const PpfBoundary* b, const double* in, double* out,
                        const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  return run_march7<double>(Diffusion7<double>{p->dt * p->D / (p->dx * p->dx)}, p->dx,
                            g, b, in, out, t, s);
}
int32_t allen_cahn3d_f32(const PpfAllenCahnParams* p, const PpfGrid* g,
                         const PpfBoundary* b, const float* in, float* out,
                         const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  AllenCahn7<float> op{(float)(p->dt * p->M * p->epsilon * p->epsilon / (p->dx * p->dx)),
                       (float)(p->dt * p->M * 16.0 * p->W)};
  return run_march7<float>(op, p->dx, g, b, in, out, t, s);
}
int32_t allen_cahn3d_f64(const PpfAllenCahnParams* p, const PpfGrid* g,
                         const PpfBoundary* b, const double* in, double* out,
                         const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  AllenCahn7<double> op{p->dt * p->M * p->epsilon * p->epsilon / (p->dx * p->dx),
                        p->dt * p->M * 16.0 * p->W};
  return run_march7<double>(op, p->dx, g, b, in, out, t, s);
}

}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_cahn_hilliard_step_f32(const PpfCahnHilliardParams* p,
                                   const PpfGrid* g, const PpfBoundary* bc,
                                   const float* in, float* out,
                                   double* mass_accum, int32_t* status,
                                   const PpfTiling* tiling, void* stream) {
  return cahn_hilliard<float>(p, g, bc, in, out, mass_accum, status, tiling, stream);
}
int32_t ppf_cahn_hilliard_step_f64(const PpfCahnHilliardParams* p,
                                   const PpfGrid* g, const PpfBoundary* bc,
                                   const double* in, double* out,
                                   double* mass_accum, int32_t* status,
                                   const PpfTiling* tiling, void* stream) {
  return cahn_hilliard<double>(p, g, bc, in, out, mass_accum, status, tiling, stream);
}

}  // extern "C"
