// 3-D explicit steps that march along z: Diffusion / Allen-Cahn (7-point)
// and Cahn-Hilliard (radius 2 through an on-chip chemical-potential tile).
//
// A CTA owns a TY x TX column of the grid and a chunk of ZC planes. Its
// z-planes (with an xy halo) are staged by TMA tensor loads into a ring of
// shared-memory slots, several planes ahead of the plane being computed, so
// HBM reads overlap the stencil; each plane is read once and written once
// (xy halos are re-read from L2). The TMA box starts 4 columns left of the
// tile (16-byte aligned); cells outside the grid arrive zero-filled and are
// rewritten with the boundary rule on edge tiles only.
//
// Reference: Field.laplacian (field.py:60-67), engine_ExplicitDiffusion
// (Engines/Diffusion.py:198-208), engine_CahnAllenExplicit
// (Engines/CahnAllen.py:128-135), engine_CahnHilliardExplicit
// (Engines/CahnHilliard.py:134-146).
#include <cmath>

#include "ppf_common.cuh"
#include "ppf_tma.cuh"

namespace ppf {
namespace {

constexpr int kThreads = 256;
constexpr int kXOff = 4;  // box starts kXOff columns left of the tile

template <typename T>
struct Diffusion7 {
  T r;
  __device__ __forceinline__ T operator()(T c, T w, T e, T n, T s, T d, T u) const {
    const T lap = (((w + e) + (n + s)) + (d + u)) - T(6) * c;
    return c + r * lap;
  }
};

template <typename T>
struct AllenCahn7 {
  T a, b;
  __device__ __forceinline__ T operator()(T c, T w, T e, T n, T s, T d, T u) const {
    const T lap = (((w + e) + (n + s)) + (d + u)) - T(6) * c;
    const T fp = c * (T(2) + c * (T(-6) + T(4) * c));
    return c + (a * lap - b * fp);
  }
};

// Shared-memory plane ring fed by TMA. Plane p (p >= pbase) lives in slot
// (p - pbase) % NS; its k-th use of the slot completes mbarrier phase k.
template <typename T, int NS>
struct PlaneRing {
  T* slots;
  uint64_t* bars;
  int slot_elems;  // elements per slot (BX * BY, padded to 128 bytes)
  int pbase;
  // p >= pbase always: unsigned arithmetic (a mask when NS is a power of two)
  __device__ T* plane(int p) const { return slots + ((unsigned)(p - pbase) % NS) * slot_elems; }
  __device__ uint64_t* bar(int p) const { return bars + (unsigned)(p - pbase) % NS; }
  __device__ uint32_t parity(int p) const { return ((unsigned)(p - pbase) / NS) & 1u; }
};

struct MarchGeom {
  int TX, TY, ZC, H;  // tile, z chunk, halo
  int BX, BY;         // TMA box (BX = TX + 2 * kXOff, BY = TY + 2H)
};

// A plane outside the grid along a non-periodic z axis is a ghost plane:
// its values follow the boundary rule (Neumann offset, Dirichlet value), so
// the fix-up writes all of it.
template <typename T>
__device__ __forceinline__ bool ghost_plane(const Geo& g, const Bc<T>& bc, int p) {
  return (unsigned)p >= (unsigned)g.n[0] && bc.type[0] != PPF_BC_PERIODIC;
}

// Issue (one thread) the load of plane p. A ghost plane is not loaded; its
// barrier phase is completed by a plain arrive instead.
template <typename T, int NS>
__device__ __forceinline__ void issue_plane(const PlaneRing<T, NS>& ring, const CUtensorMap* map,
                                            const Geo& g, const Bc<T>& bc, const MarchGeom& m,
                                            int x0, int y0, int p) {
  uint64_t* b = ring.bar(p);
  const int nz = g.n[0];
  if (ghost_plane(g, bc, p)) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
    return;
  }
  const int pz = wrap_index(p, nz);
  fence_proxy_async();
  mbar_expect_tx(b, (uint32_t)(m.BX * m.BY * sizeof(T)));
  tma_load_3d(ring.plane(p), map, x0 - kXOff, y0 - m.H, pz, b);
}

// The cells of a CTA's W x Hh window (W = TX + 2H, Hh = TY + 2H) that lie
// outside the grid: cl / cr columns on the left / right, rt / rb rows at the
// top / bottom, enumerated as the full rows first, then the outside columns
// of the remaining rows.
struct EdgeSet {
  int W, Hh, cl, cr, rt, rb, nrow, ncol, count;
};

__device__ __forceinline__ EdgeSet edge_set(const MarchGeom& m, const Geo& g, int x0, int y0) {
  EdgeSet E;
  E.W = m.TX + 2 * m.H;
  E.Hh = m.TY + 2 * m.H;
  E.cl = min(E.W, max(0, m.H - x0));
  E.cr = min(E.W - E.cl, max(0, x0 - m.H + E.W - g.n[2]));
  E.rt = min(E.Hh, max(0, m.H - y0));
  E.rb = min(E.Hh - E.rt, max(0, y0 - m.H + E.Hh - g.n[1]));
  E.nrow = (E.rt + E.rb) * E.W;
  E.ncol = E.cl + E.cr;
  E.count = E.nrow + (E.Hh - E.rt - E.rb) * E.ncol;
  return E;
}

// Window coordinates (ly, lx) of edge cell e < E.count.
__device__ __forceinline__ void edge_cell(const EdgeSet& E, int e, int& ly, int& lx) {
  if (e < E.nrow) {
    const int r = e / E.W;
    ly = r < E.rt ? r : E.Hh - E.rb + (r - E.rt);
    lx = e - r * E.W;
  } else {
    const int e2 = e - E.nrow;
    const int r = e2 / E.ncol, c = e2 - r * E.ncol;
    ly = E.rt + r;
    lx = c < E.cl ? c : E.W - E.cr + (c - E.cl);
  }
}

// Edge cells per thread held in registers between the fetch of a plane's
// edge values and their store into its slot.
constexpr int kEdgeRegs = 2;

// Fetch (boundary rule, global loads) the edge values of plane p into
// registers: issued one plane ahead, the loads overlap the stencil of the
// current plane.
template <typename T>
__device__ __forceinline__ void edge_load(const EdgeSet& E, const T* __restrict__ in,
                                          const Geo& g, const Bc<T>& bc, const MarchGeom& m,
                                          int x0, int y0, int p, T (&v)[kEdgeRegs]) {
  const int tid = threadIdx.x + 32 * threadIdx.y;
#pragma unroll
  for (int k = 0; k < kEdgeRegs; ++k) {
    const int e = tid + k * kThreads;
    if (e < E.count) {
      int ly, lx;
      edge_cell(E, e, ly, lx);
      v[k] = fetch<T, 3>(in, g, bc, 0, p, y0 - m.H + ly, x0 - m.H + lx);
    }
  }
}

// Store the edge values of plane p (after its TMA load landed); cells
// beyond kEdgeRegs per thread are fetched here.
template <typename T, int NS>
__device__ __forceinline__ void edge_store(const EdgeSet& E, const PlaneRing<T, NS>& ring,
                                           const T* __restrict__ in, const Geo& g,
                                           const Bc<T>& bc, const MarchGeom& m, int x0, int y0,
                                           int p, const T (&v)[kEdgeRegs]) {
  T* dst = ring.plane(p) + (kXOff - m.H);
  const int tid = threadIdx.x + 32 * threadIdx.y;
#pragma unroll
  for (int k = 0; k < kEdgeRegs; ++k) {
    const int e = tid + k * kThreads;
    if (e < E.count) {
      int ly, lx;
      edge_cell(E, e, ly, lx);
      dst[ly * m.BX + lx] = v[k];
    }
  }
  for (int e = tid + kEdgeRegs * kThreads; e < E.count; e += kThreads) {
    int ly, lx;
    edge_cell(E, e, ly, lx);
    dst[ly * m.BX + lx] = fetch<T, 3>(in, g, bc, 0, p, y0 - m.H + ly, x0 - m.H + lx);
  }
}

// Rewrite the cells of plane p that the TMA box could not supply: the edge
// cells of an edge tile, or the whole of a ghost plane, by the generic
// boundary rule.
template <typename T, int NS>
__device__ __forceinline__ void fixup_plane(const PlaneRing<T, NS>& ring, const T* __restrict__ in,
                                            const Geo& g, const Bc<T>& bc, const MarchGeom& m,
                                            int x0, int y0, int p, bool xy_edge) {
  const bool zfixed = ghost_plane(g, bc, p);
  if (!xy_edge && !zfixed) return;
  T* dst = ring.plane(p);
  const int W = m.TX + 2 * m.H, Hh = m.TY + 2 * m.H;
  if (zfixed) {
    for (int ly = threadIdx.y; ly < Hh; ly += kThreads / 32) {
      const int gy = y0 - m.H + ly;
      for (int lx = threadIdx.x; lx < W; lx += 32) {
        const int gx = x0 - m.H + lx;
        dst[ly * m.BX + (gx - x0 + kXOff)] = fetch<T, 3>(in, g, bc, 0, p, gy, gx);
      }
    }
    return;
  }
  const EdgeSet E = edge_set(m, g, x0, y0);
  for (int e = threadIdx.x + 32 * threadIdx.y; e < E.count; e += kThreads) {
    int ly, lx;
    edge_cell(E, e, ly, lx);
    dst[ly * m.BX + lx + (kXOff - m.H)] =
        fetch<T, 3>(in, g, bc, 0, p, y0 - m.H + ly, x0 - m.H + lx);
  }
}

// Asynchronous copy of one element from global to shared memory (the
// issuing thread waits for its copies with cp_async_wait_all).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src),
               "n"((int)sizeof(T))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Bounded wait by every thread; returns false (uniformly) if any timed out.
__device__ __forceinline__ bool wait_all(uint64_t* bar, uint32_t parity, int* abort_flag) {
  if (!mbar_wait(bar, parity)) *abort_flag = 1;
  __syncthreads();
  return *abort_flag == 0;
}

template <typename T>
__device__ __forceinline__ void report_timeout(int* status) {
  if (threadIdx.x == 0 && threadIdx.y == 0) atomicOr(status, PPF_STATUS_TIMEOUT);
}

// After a timeout: wait (bounded) for every plane still in flight so that no
// TMA write lands in shared memory after the CTA has exited.
template <typename T, int NS>
__device__ void drain(const PlaneRing<T, NS>& ring, int first, int last) {
  if (threadIdx.x == 0 && threadIdx.y == 0)
    for (int p = first; p <= last; ++p) mbar_wait(ring.bar(p), ring.parity(p));
  __syncthreads();
}

// First 128-byte aligned address at or after p (the dynamic shared memory
// base). The offset is added to p itself, not to an integer copy of it, so
// the compiler keeps the shared address space and emits shared loads.
template <typename T>
__device__ __forceinline__ T* align128(unsigned char* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  return reinterpret_cast<T*>(p + ((128u - (a & 127u)) & 127u));
}

// ------------------------------------------------------------- 7-point
constexpr int kNS7 = 5;  // planes z-1, z, z+1 in use; z+2, z+3 in flight

template <typename T, typename Op>
__global__ void __launch_bounds__(kThreads)
    march7_kernel(const __grid_constant__ CUtensorMap map, Op op, Geo g, Bc<T> bc,
                  const T* __restrict__ in, T* __restrict__ out, MarchGeom m, int slot_elems,
                  int* status) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[kNS7];
  __shared__ int abort_flag;
  const int x0 = blockIdx.x * m.TX, y0 = blockIdx.y * m.TY, z0 = blockIdx.z * m.ZC;
  const int nz = g.n[0], ny = g.n[1], nx = g.n[2];
  const int z1 = min(z0 + m.ZC, nz);
  const bool xy_edge = x0 - 1 < 0 || y0 - 1 < 0 || x0 + m.TX + 1 > nx || y0 + m.TY + 1 > ny ||
                       x0 - kXOff < 0 || x0 + m.TX + kXOff > nx;
  PlaneRing<T, kNS7> ring{align128<T>(smem_raw), bars, slot_elems, z0 - 1};
  const bool leader = threadIdx.x == 0 && threadIdx.y == 0;

  if (leader) {
    for (int i = 0; i < kNS7; ++i) mbar_init(&bars[i], 1);
    mbar_init_fence();
    abort_flag = 0;
  }
  __syncthreads();
  pdl_wait();
  pdl_launch_next();
  const int last = z1;  // last plane needed
  if (leader)
    for (int p = z0 - 1; p <= min(z0 + 2, last); ++p) issue_plane(ring, &map, g, bc, m, x0, y0, p);
  int issued = min(z0 + 2, last);

  for (int p = z0 - 1; p <= z0; ++p) {
    if (!wait_all(ring.bar(p), ring.parity(p), &abort_flag)) {
      report_timeout<T>(status);
      drain(ring, p, issued);
      return;
    }
    fixup_plane(ring, in, g, bc, m, x0, y0, p, xy_edge);
  }
  const int W = m.BX;
  for (int z = z0; z < z1; ++z) {
    if (leader && z + 3 <= last) {
      issue_plane(ring, &map, g, bc, m, x0, y0, z + 3);
      issued = z + 3;
    }
    if (!wait_all(ring.bar(z + 1), ring.parity(z + 1), &abort_flag)) {
      report_timeout<T>(status);
      if (leader) issued = min(z + 3, last);
      drain(ring, z + 1, min(z + 3, last));
      return;
    }
    fixup_plane(ring, in, g, bc, m, x0, y0, z + 1, xy_edge);
    __syncthreads();
    const T* pd = ring.plane(z - 1);
    const T* pc = ring.plane(z);
    const T* pu = ring.plane(z + 1);
    for (int ly = 1 + threadIdx.y; ly <= m.TY; ly += kThreads / 32) {
      const int gy = y0 + ly - 1;
      if (gy >= ny) break;
      T* orow = out + (int64_t)z * g.plane + (int64_t)gy * g.pitch;
      for (int lx = threadIdx.x; lx < m.TX; lx += 32) {
        const int gx = x0 + lx;
        if (gx >= nx) break;
        const int i = ly * W + lx + kXOff;
        orow[gx] = op(pc[i], pc[i - 1], pc[i + 1], pc[i - W], pc[i + W], pd[i], pu[i]);
      }
    }
    __syncthreads();
  }
}

// Lean 7-point kernel (the default tile): 32 x 32 cells, 256 threads, each
// thread owns the 4 xy-columns (ty + 8q, tx) and keeps c(z - 1), c(z) of
// each in registers while marching along z, so a cell reads only its four
// xy neighbours and the new plane's centre from shared memory; every shared
// index is a compile-time offset from one per-thread base and there is one
// block barrier per plane.
constexpr int kLTX = 32;
constexpr int kLTY = 32;
constexpr int kLQ = kLTY / 8;
constexpr int kLW = kLTX + 2 * kXOff;  // TMA box width
constexpr int kNSL = 6;                // planes z, z+1 read; z+2 .. z+4 in flight

template <typename T, typename Op, bool EDGE_COPY>
__global__ void __launch_bounds__(kThreads)
    march7_lean_kernel(const __grid_constant__ CUtensorMap map, Op op, Geo g, Bc<T> bc,
                       const T* __restrict__ in, T* __restrict__ out, MarchGeom m,
                       int slot_elems, int* status) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[kNSL];
  __shared__ int abort_flag;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * kLTX, y0 = blockIdx.y * kLTY, z0 = blockIdx.z * m.ZC;
  const int nz = g.n[0], ny = g.n[1], nx = g.n[2];
  const int z1 = min(z0 + m.ZC, nz);
  const bool xy_edge = x0 - kXOff < 0 || y0 - 1 < 0 || x0 + kLTX + kXOff > nx ||
                       y0 + kLTY + 1 > ny;
  PlaneRing<T, kNSL> ring{align128<T>(smem_raw), bars, slot_elems, z0 - 1};
  const bool leader = tx == 0 && ty == 0;

  if (leader) {
    for (int i = 0; i < kNSL; ++i) mbar_init(&bars[i], 1);
    mbar_init_fence();
    abort_flag = 0;
  }
  __syncthreads();
  pdl_wait();
  pdl_launch_next();
  const int last = z1;  // plane z1 is the upper neighbour of the last plane
  if (leader)
    for (int p = z0 - 1; p <= min(z0 + kNSL - 3, last); ++p)
      issue_plane(ring, &map, g, bc, m, x0, y0, p);
  for (int p = z0 - 1; p <= z0; ++p) {
    if (!wait_all(ring.bar(p), ring.parity(p), &abort_flag)) {
      report_timeout<T>(status);
      drain(ring, p, min(z0 + kNSL - 3, last));
      return;
    }
    fixup_plane(ring, in, g, bc, m, x0, y0, p, xy_edge);
  }
  __syncthreads();

  const int ci = (ty + 1) * kLW + tx + kXOff;
  T cm[kLQ], c0[kLQ];
  {
    const T* Pm = ring.plane(z0 - 1);
    const T* P0 = ring.plane(z0);
#pragma unroll
    for (int q = 0; q < kLQ; ++q) {
      cm[q] = Pm[ci + q * 8 * kLW];
      c0[q] = P0[ci + q * 8 * kLW];
    }
  }
  T* optr = out + (int64_t)z0 * g.plane + (int64_t)(y0 + ty) * g.pitch + x0 + tx;
  const int64_t qstride = (int64_t)8 * g.pitch;
  const bool xin = x0 + tx < nx;
  int nq = 0;
#pragma unroll
  for (int q = 0; q < kLQ; ++q) nq += (xin && y0 + ty + 8 * q < ny) ? 1 : 0;
  const bool full = x0 + kLTX <= nx && y0 + kLTY <= ny;

  // Edge tiles of a grid periodic along y and x (window cells outside the
  // grid are plain copies of cells on the far side, at most one per thread,
  // plane offsets below 2^31): thread tid copies window cell tid's source,
  // found once here, into each plane's slot.
  // EDGE_COPY: the instantiation for grids with many edge tiles (the copy
  // costs eight registers a thread, one CTA per SM less).
  int e_dst = -1, e_src = 0;
  bool async_tile = false;
  if (EDGE_COPY && xy_edge && bc.type[1] == PPF_BC_PERIODIC && bc.type[2] == PPF_BC_PERIODIC &&
      (int64_t)ny * g.pitch < (1LL << 31)) {
    const EdgeSet E = edge_set(m, g, x0, y0);
    async_tile = E.count <= kThreads;
    const int tid = tx + 32 * ty;
    if (async_tile && tid < E.count) {
      int ly, lx;
      edge_cell(E, tid, ly, lx);
      e_dst = ly * m.BX + lx + (kXOff - m.H);
      e_src = wrap_index(y0 - m.H + ly, ny) * (int)g.pitch + wrap_index(x0 - m.H + lx, nx);
    }
  }

  for (int z = z0; z < z1; ++z) {
    // plane z + kNSL - 2 takes the slot of plane z - 2, last read in
    // iteration z - 2 (plane p is read in iterations p - 1 and p), which
    // every thread finished before the barrier of iteration z - 1
    if (leader && z + kNSL - 2 <= last) issue_plane(ring, &map, g, bc, m, x0, y0, z + kNSL - 2);
    if (!wait_all(ring.bar(z + 1), ring.parity(z + 1), &abort_flag)) {
      report_timeout<T>(status);
      drain(ring, z + 1, min(z + kNSL - 2, last));
      return;
    }
    // (no register prefetch of the edge values here: its registers cost
    // this kernel more occupancy than the hidden loads gain)
    const bool zghost = ghost_plane(g, bc, z + 1);
    const bool async_edge = async_tile && !zghost;
    if (zghost || (xy_edge && !async_edge)) {
      fixup_plane(ring, in, g, bc, m, x0, y0, z + 1, xy_edge);
      __syncthreads();
    }
    if (async_edge) {
      // Iteration z reads only the own (inside) cells of plane z + 1, its
      // cells outside the grid from iteration z + 1 on, after that
      // iteration's barrier: they are copied into the slot (which its TMA
      // load has filled) asynchronously during this plane's stencil, each
      // thread waiting for its copy at the end of the iteration.
      if (e_dst >= 0)
        cp_async_elem(ring.plane(z + 1) + e_dst,
                      in + (int64_t)wrap_index(z + 1, nz) * g.plane + e_src);
      cp_async_commit();
    }
    const T* P0 = ring.plane(z);
    const T* P1 = ring.plane(z + 1);
#pragma unroll
    for (int q = 0; q < kLQ; ++q) {
      const int i = ci + q * 8 * kLW;
      const T cp = P1[i];
      const T v = op(c0[q], P0[i - 1], P0[i + 1], P0[i - kLW], P0[i + kLW], cm[q], cp);
      if (full || q < nq) optr[q * qstride] = v;
      cm[q] = c0[q];
      c0[q] = cp;
    }
    optr += g.plane;
    if (async_edge) cp_async_wait_all();
  }
}

// ------------------------------------------------------------- Cahn-Hilliard
// mu~ = -(eps^2/dx^2) lap'(c) + f'(c), lap' the unscaled 7-point sum;
// c' = c + sum over the 6 faces of F = a (mu~_nbr - mu~_c), a = dt M/dx^2.
// With QUANT each face flux is rounded to a multiple of q (a power of two).
// F(A->B) = -F(B->A) bit for bit (the same mu~ values enter both cells and
// rounding to nearest is odd-symmetric), so the float field conserves its
// sum exactly while every value stays a multiple of q below 2^24 q.
template <typename T>
struct ChCoef {
  T kap;         // eps^2/dx^2
  T a;           // dt*M/dx^2
  T aiq;         // a / q (QUANT only; exact: q is a power of two)
  T q, iq;       // quantum and its inverse (QUANT only)
  T range;       // 2^24 q: |c| beyond this loses exactness (QUANT only)
  int centered;  // field holds u = c - 1/2
};

template <typename T>
__device__ __forceinline__ T ch_mu(const ChCoef<T>& k, T c, T w, T e, T n, T s, T d, T u) {
  const T lap = (((w + e) + (n + s)) + (d + u)) - T(6) * c;
  // 4c^3 - 6c^2 + 2c, or in the centered variable 4u^3 - u
  const T fp = k.centered ? c * (T(4) * c * c - T(1)) : c * (T(2) + c * (T(-6) + T(4) * c));
  return fp - k.kap * lap;
}

template <typename T, bool QUANT>
__device__ __forceinline__ T ch_flux(const ChCoef<T>& k, T mn, T mc) {
  // (a d) / q == (a / q) d bit for bit: scaling by a power of two is exact
  if (QUANT) return rint(k.aiq * (mn - mc)) * k.q;
  return k.a * (mn - mc);
}

constexpr int kNSC = 7;  // c planes z..z+2 read, z+3 .. z+5 in flight
constexpr int kMuSlots = 3;  // mu planes z - 1, z, z + 1
// Cahn-Hilliard tile: 32 x 32 cells, 256 threads; thread (tx, ty) owns the
// kCQ = 4 xy-columns (ty + 8q, tx) and keeps, per column, c(z), c(z+1),
// mu(z) and the flux through the face below plane z in registers while
// marching along z (the flux through a face is computed once: the cell
// above takes it negated, bit for bit). mu of the tile plus a one-cell ring
// lives in a three-plane shared ring for the xy fluxes (one block barrier
// per plane: the one that publishes mu(z + 1)); the kRingN ring
// positions are computed by threads 0..kRingN-1. Every shared index is a
// compile-time offset from a per-thread base.
constexpr int kCTX = 32;
constexpr int kCTY = 32;
constexpr int kCQ = kCTY / 8;
constexpr int kCW = kCTX + 2 * kXOff;     // c plane row length (TMA box width)
constexpr int kCH = kCTY + 4;             // c plane rows (halo 2)
constexpr int kCSlot = kCW * kCH;         // 1440 elements, a multiple of 128 bytes
constexpr int kMW = kCTX + 2;
constexpr int kMH = kCTY + 2;
constexpr int kMN = kMW * kMH;
constexpr int kRingN = kMN - kCTX * kCTY;  // 132

// Ring position i -> mu-region coordinates (ly, lx) on the border.
__device__ __forceinline__ void ring_pos(int i, int& ly, int& lx) {
  if (i < kMW) {
    ly = 0;
    lx = i;
  } else if (i < 2 * kMW) {
    ly = kMH - 1;
    lx = i - kMW;
  } else if (i < 2 * kMW + kCTY) {
    ly = 1 + (i - 2 * kMW);
    lx = 0;
  } else {
    ly = 1 + (i - 2 * kMW - kCTY);
    lx = kMW - 1;
  }
}

template <typename T, bool QUANT>
__global__ void __launch_bounds__(kThreads)
    cahn_hilliard_kernel(const __grid_constant__ CUtensorMap map, ChCoef<T> k, Geo g, Bc<T> bc,
                         const T* __restrict__ in, T* __restrict__ out, double* __restrict__ mass,
                         int* __restrict__ status, MarchGeom m, int slot_elems,
                         int* __restrict__ lib_status) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[kNSC];
  __shared__ int abort_flag;
  __shared__ double red[kThreads / 32];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + 32 * ty;
  const int x0 = blockIdx.x * kCTX, y0 = blockIdx.y * kCTY, z0 = blockIdx.z * m.ZC;
  const int nz = g.n[0], ny = g.n[1], nx = g.n[2];
  const int z1 = min(z0 + m.ZC, nz);
  const bool xy_edge = x0 - kXOff < 0 || y0 - 2 < 0 || x0 + kCTX + kXOff > nx ||
                       y0 + kCTY + 2 > ny;
  PlaneRing<T, kNSC> ring{align128<T>(smem_raw), bars, kCSlot, z0 - 2};
  // kMuSlots mu planes: in iteration z a thread writes mu(z + 1) while
  // others may still read mu(z - 1) (nothing but the one barrier per plane
  // orders the iterations), so mu(z - 1), mu(z), mu(z + 1) need three slots
  T* const mring = ring.slots + kNSC * kCSlot;
  const bool leader = tid == 0;
  (void)slot_elems;

  // own cells q: c-plane index ci + q * 8 * kCW, mu-plane index mi + q * 8 * kMW
  const int ci = (ty + 2) * kCW + tx + kXOff;
  const int mi = (ty + 1) * kMW + tx + 1;
  const bool has_ring = tid < kRingN;
  int rci = 0, rmi = 0;
  if (has_ring) {
    int ly, lx;
    ring_pos(tid, ly, lx);
    rci = (ly + 1) * kCW + lx + (kXOff - 1);
    rmi = ly * kMW + lx;
  }

  if (leader) {
    for (int i = 0; i < kNSC; ++i) mbar_init(&bars[i], 1);
    mbar_init_fence();
    abort_flag = 0;
  }
  __syncthreads();
  pdl_wait();
  pdl_launch_next();
  const int last = z1 + 1;
  if (leader)
    for (int p = z0 - 2; p <= min(z0 + kNSC - 3, last); ++p)
      issue_plane(ring, &map, g, bc, m, x0, y0, p);
  for (int p = z0 - 2; p <= z0 + 1; ++p) {
    if (!wait_all(ring.bar(p), ring.parity(p), &abort_flag)) {
      report_timeout<T>(lib_status);
      drain(ring, p, min(z0 + kNSC - 3, last));
      return;
    }
    fixup_plane(ring, in, g, bc, m, x0, y0, p, xy_edge);
  }
  __syncthreads();

  auto mu_at = [&](const T* cd, const T* cc, const T* cu, int i) {
    return ch_mu(k, cc[i], cc[i - 1], cc[i + 1], cc[i - kCW], cc[i + kCW], cd[i], cu[i]);
  };
  T c0[kCQ], c1[kCQ], mu0[kCQ], fup[kCQ];
  {
    const T* Pm2 = ring.plane(z0 - 2);
    const T* Pm1 = ring.plane(z0 - 1);
    const T* P0 = ring.plane(z0);
    const T* P1 = ring.plane(z0 + 1);
    T* M0 = mring;
#pragma unroll
    for (int q = 0; q < kCQ; ++q) {
      const int i = ci + q * 8 * kCW;
      const T mum = mu_at(Pm2, Pm1, P0, i);
      mu0[q] = mu_at(Pm1, P0, P1, i);
      M0[mi + q * 8 * kMW] = mu0[q];
      c0[q] = P0[i];
      c1[q] = P1[i];
      // flux through the face below z0, stored negated as "flux into the
      // cell below from above": the loop takes fd = -fup
      fup[q] = -ch_flux<T, QUANT>(k, mum, mu0[q]);
    }
    if (has_ring) M0[rmi] = mu_at(Pm1, P0, P1, rci);
  }
  // the first iteration's load goes into the slot of plane z0 - 2, read
  // just above
  __syncthreads();

  T* optr = out + (int64_t)z0 * g.plane + (int64_t)(y0 + ty) * g.pitch + x0 + tx;
  const int64_t qstride = (int64_t)8 * g.pitch;
  const bool xin = x0 + tx < nx;
  int nq = 0;  // own rows inside the grid: rows ty + 8q < ny - y0
#pragma unroll
  for (int q = 0; q < kCQ; ++q) nq += (xin && y0 + ty + 8 * q < ny) ? 1 : 0;
  // CTA-uniform: the whole tile lies inside the grid (no per-cell checks)
  const bool full = x0 + kCTX <= nx && y0 + kCTY <= ny;

  long long acc_q = 0;
  double acc = 0.0;
  T vmax = T(0), vsum = T(0);
  int m0i = 0;  // mu slot of plane z
  // edge tiles: the boundary-rule values of plane z + 2 are fetched into
  // registers during iteration z - 1
  const EdgeSet E = edge_set(m, g, x0, y0);
  const bool has_edge = xy_edge && E.count > 0;
  T pre[kEdgeRegs];
  if (has_edge && z0 + 2 <= last && !ghost_plane(g, bc, z0 + 2))
    edge_load(E, in, g, bc, m, x0, y0, z0 + 2, pre);
  for (int z = z0; z < z1; ++z) {
    // plane z + kNSC - 2 reuses the slot of plane z - 2, last read in
    // iteration z - 2 (c plane p is read in iterations p - 2 .. p), before
    // the barriers of iteration z - 1
    if (leader && z + kNSC - 2 <= last) issue_plane(ring, &map, g, bc, m, x0, y0, z + kNSC - 2);
    // every thread waits for plane z + 2 itself; a timeout is acted on, by
    // all threads alike, after the barrier below
    if (!mbar_wait(ring.bar(z + 2), ring.parity(z + 2))) abort_flag = 1;
    if (ghost_plane(g, bc, z + 2)) {
      fixup_plane(ring, in, g, bc, m, x0, y0, z + 2, xy_edge);
      __syncthreads();
    } else if (has_edge) {
      edge_store(E, ring, in, g, bc, m, x0, y0, z + 2, pre);
      __syncthreads();
    }
    if (has_edge && z + 3 <= last && !ghost_plane(g, bc, z + 3))
      edge_load(E, in, g, bc, m, x0, y0, z + 3, pre);
    const T* P0 = ring.plane(z);
    const T* P1 = ring.plane(z + 1);
    const T* P2 = ring.plane(z + 2);
    const int m1i = m0i == kMuSlots - 1 ? 0 : m0i + 1;
    T* M1 = mring + m1i * kMN;
    T c2[kCQ], mup[kCQ];
#pragma unroll
    for (int q = 0; q < kCQ; ++q) {
      const int i = ci + q * 8 * kCW;
      c2[q] = P2[i];
      mup[q] = ch_mu(k, c1[q], P1[i - 1], P1[i + 1], P1[i - kCW], P1[i + kCW], c0[q], c2[q]);
      M1[mi + q * 8 * kMW] = mup[q];
    }
    if (has_ring) M1[rmi] = mu_at(P0, P1, P2, rci);
    __syncthreads();
    if (abort_flag) {
      report_timeout<T>(lib_status);
      drain(ring, z + 2, min(z + kNSC - 2, last));
      return;
    }
    const T* M0 = mring + m0i * kMN;
    m0i = m1i;
    int32_t quanta = 0;
#pragma unroll
    for (int q = 0; q < kCQ; ++q) {
      const int i = mi + q * 8 * kMW;
      const T m0 = mu0[q];
      const T fw = ch_flux<T, QUANT>(k, M0[i - 1], m0);
      const T fe = ch_flux<T, QUANT>(k, M0[i + 1], m0);
      const T fn = ch_flux<T, QUANT>(k, M0[i - kMW], m0);
      const T fs = ch_flux<T, QUANT>(k, M0[i + kMW], m0);
      const T fu = ch_flux<T, QUANT>(k, mup[q], m0);
      const T fd = -fup[q];
      const T v = c0[q] + (((fw + fe) + (fn + fs)) + (fd + fu));
      if (full || q < nq) {
        optr[q * qstride] = v;
        if (QUANT) quanta += __float2int_rn((float)(v * k.iq));  // exact: |v / q| < 2^24
        else acc += (double)v;
        vmax = fmax(vmax, fabs(v));
        vsum += v;
      }
      c0[q] = c1[q];
      c1[q] = c2[q];
      mu0[q] = mup[q];
      fup[q] = fu;
    }
    acc_q += quanta;
    optr += g.plane;
  }
  int flags = 0;
  if (QUANT && !(vmax < k.range)) flags |= PPF_STATUS_RANGE;
  if (!isfinite(vsum) || !isfinite(vmax)) flags |= PPF_STATUS_NONFINITE;
  if (status && flags) atomicOr(status, flags);
  if (mass) {
    // QUANT: exact integer count of quanta (|sum| < 2^53), scaled by q at
    // the end: the total is the same whatever order the CTAs add in.
    double v = QUANT ? (double)acc_q : acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (tx == 0) red[ty] = v;
    __syncthreads();
    if (ty == 0) {
      double s = tx < kThreads / 32 ? red[tx] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (tx == 0) atomicAdd(mass, QUANT ? s * (double)k.q : s);
    }
  }
}

// ------------------------------------------------------------- host side
template <typename T>
int32_t plan3d(const PpfTiling* t, const Geo& g, int halo, int nslots, int mu_planes,
               MarchGeom* m, int* slot_elems, size_t* smem) {
  m->TX = t && t->tile_x ? t->tile_x : 64;
  m->TY = t && t->tile_y ? t->tile_y : 16;
  m->H = halo;
  if (t && t->depth > 1)
    return fail(PPF_ERR_UNSUPPORTED, "3-D steps advance one step per pass (depth=%d)", t->depth);
  if (m->TX < 4 || m->TX > 256 - 2 * kXOff || (m->TX % 4) != 0 || m->TY < 1 ||
      m->TY + 2 * halo > 256)
    return fail(PPF_ERR_INVALID, "tile %dx%d invalid (tile_x multiple of 4, <= %d)", m->TX,
                m->TY, 256 - 2 * kXOff);
  m->BX = m->TX + 2 * kXOff;
  m->BY = m->TY + 2 * halo;
  if (t && t->zchunk < 0) return fail(PPF_ERR_INVALID, "zchunk must be >= 0");
  m->ZC = 0;  // set by the caller (zchunk_of)
  const size_t slot_bytes = ((size_t)m->BX * m->BY * sizeof(T) + 127) / 128 * 128;
  *slot_elems = (int)(slot_bytes / sizeof(T));
  *smem = 128 + (size_t)nslots * slot_bytes +
          (size_t)mu_planes * (m->TX + 2) * (m->TY + 2) * sizeof(T);
  if (*smem > 200 * 1024)
    return fail(PPF_ERR_INVALID, "tile needs %zu bytes of shared memory", *smem);
  return PPF_OK;
}

// Planes per CTA along z when the caller leaves it open: short chunks (many
// CTAs in flight over a compact stretch of z) measured fastest on GB300 for
// both 3-D kernels (384^3 and 512^3: 8-16 planes beat 32-64 by 1.3-1.9x, and
// sizing the chunks to one wave of CTAs was slower still).
constexpr int kDefaultZChunk = 12;

int zchunk_of(const PpfTiling* t, const Geo& g) {
  const int zc = t && t->zchunk > 0 ? t->zchunk : kDefaultZChunk;
  return zc < g.n[0] ? zc : g.n[0];
}

template <typename T>
int32_t plane_map(CUtensorMap* map, const T* base, const Geo& g, const MarchGeom& m) {
  const uint64_t dims[3] = {(uint64_t)g.n[2], (uint64_t)g.n[1], (uint64_t)g.n[0]};
  const uint64_t strides[2] = {(uint64_t)g.pitch * sizeof(T), (uint64_t)g.plane * sizeof(T)};
  const uint32_t box[3] = {(uint32_t)m.BX, (uint32_t)m.BY, 1u};
  return tensor_map(map, base, (int)sizeof(T), 3, dims, strides, box);
}

// A 2-D grid runs as a single-plane 3-D grid with a periodic z axis (the
// z neighbours are the cell itself and cancel in the Laplacian).
int32_t as3d(const PpfGrid* in, const PpfBoundary* bin, PpfGrid* g3, PpfBoundary* b3) {
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
int32_t run_march7(Op op, double dx, const PpfGrid* grid, const PpfBoundary* b, const T* in,
                   T* out, const PpfTiling* tiling, void* stream) {
  Geo g;
  int32_t rc = make_geo(grid, 3, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (in == out) return fail(PPF_ERR_INVALID, "in and out must differ");
  Bc<T> bc;
  if ((rc = make_bc<T>(b, g, dx, 1, 1, &bc))) return rc;
  MarchGeom m;
  int slot_elems;
  size_t smem;
  int* st = status_ptr();
  if (!st) return fail(PPF_ERR_CUDA, "status word unavailable");
  const bool lean = !tiling || ((tiling->tile_x == 0 || tiling->tile_x == kLTX) &&
                                (tiling->tile_y == 0 || tiling->tile_y == kLTY));
  if (lean) {
    PpfTiling lt{};
    lt.depth = tiling ? tiling->depth : 0;
    lt.tile_x = kLTX;
    lt.tile_y = kLTY;
    if ((rc = plan3d<T>(&lt, g, 1, kNSL, 0, &m, &slot_elems, &smem))) return rc;
    CUtensorMap map;
    if ((rc = plane_map<T>(&map, in, g, m))) return rc;
    // periodic in y and x with a quarter or more of the tiles on an edge
    // (384^3 and below): the kernel that copies the edge cells
    // asynchronously (256^3 43.8 -> 39.5 us per step, 384^3 108.9 -> 104.8;
    // 512^3 222.0 against 224.4 with it)
    const long long tx_n = (g.n[2] + kLTX - 1) / kLTX, ty_n = (g.n[1] + kLTY - 1) / kLTY;
    const long long inner = (tx_n > 2 ? tx_n - 2 : 0) * (ty_n > 2 ? ty_n - 2 : 0);
    const bool edge_copy = bc.type[1] == PPF_BC_PERIODIC && bc.type[2] == PPF_BC_PERIODIC &&
                           4 * (tx_n * ty_n - inner) >= tx_n * ty_n;
    auto kern = edge_copy ? march7_lean_kernel<T, Op, true> : march7_lean_kernel<T, Op, false>;
    PPF_TRY_CUDA(allow_smem(kern, smem));
    m.ZC = zchunk_of(tiling, g);
    dim3 gd((g.n[2] + kLTX - 1) / kLTX, (g.n[1] + kLTY - 1) / kLTY, (g.n[0] + m.ZC - 1) / m.ZC);
    PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream,
                        tiling && tiling->pdl, map, op, g, bc, in, out, m, slot_elems, st));
    return PPF_OK;
  }
  if ((rc = plan3d<T>(tiling, g, 1, kNS7, 0, &m, &slot_elems, &smem))) return rc;
  m.ZC = zchunk_of(tiling, g);
  CUtensorMap map;
  if ((rc = plane_map<T>(&map, in, g, m))) return rc;
  auto kern = march7_kernel<T, Op>;
  PPF_TRY_CUDA(allow_smem(kern, smem));
  dim3 gd((g.n[2] + m.TX - 1) / m.TX, (g.n[1] + m.TY - 1) / m.TY, (g.n[0] + m.ZC - 1) / m.ZC);
  PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream,
                      tiling && tiling->pdl, map, op, g, bc, in, out, m, slot_elems, st));
  return PPF_OK;
}

template <typename T>
int32_t cahn_hilliard(const PpfCahnHilliardParams* p, const PpfGrid* grid_in,
                      const PpfBoundary* b_in, const T* in, T* out, double* mass,
                      int32_t* status, const PpfTiling* tiling, void* stream) {
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
      return fail(PPF_ERR_UNSUPPORTED, "Cahn-Hilliard supports PERIODIC and NEUMANN axes only");
    if (b.type[a] == PPF_BC_NEUMANN && (b.value[0][a][0] != 0.0 || b.value[0][a][1] != 0.0))
      return fail(PPF_ERR_UNSUPPORTED, "Cahn-Hilliard NEUMANN axes must be no-flux (gradient 0)");
  }
  Bc<T> bc;
  if ((rc = make_bc<T>(&b, g, p->dx, 1, 2, &bc))) return rc;
  MarchGeom m;
  int slot_elems;
  size_t smem;
  if (tiling && ((tiling->tile_x && tiling->tile_x != kCTX) ||
                 (tiling->tile_y && tiling->tile_y != kCTY)))
    return fail(PPF_ERR_UNSUPPORTED, "Cahn-Hilliard tiles are %dx%d", kCTX, kCTY);
  PpfTiling ct{};
  ct.depth = tiling ? tiling->depth : 0;
  ct.tile_x = kCTX;
  ct.tile_y = kCTY;
  if ((rc = plan3d<T>(&ct, g, 2, kNSC, kMuSlots, &m, &slot_elems, &smem))) return rc;
  if (slot_elems != kCSlot || m.BX != kCW || m.BY != kCH)
    return fail(PPF_ERR_INVALID, "Cahn-Hilliard plane slot mismatch");
  ChCoef<T> k;
  k.kap = (T)(p->epsilon * p->epsilon / (p->dx * p->dx));
  k.a = (T)(p->dt * p->M / (p->dx * p->dx));
  const bool quant = p->quantum > 0;
  if (quant) {
    int e;
    const double mant = std::frexp(p->quantum, &e);
    if (mant != 0.5 || sizeof(T) != 4)
      return fail(PPF_ERR_INVALID, "quantum must be a power of two and needs the float path");
  }
  k.q = (T)(quant ? p->quantum : 0.0);
  k.iq = (T)(quant ? 1.0 / p->quantum : 0.0);
  k.aiq = (T)(quant ? (double)k.a * (1.0 / p->quantum) : 0.0);
  k.range = (T)(quant ? std::ldexp(p->quantum, 24) : 0.0);
  if (p->centered != 0 && p->centered != 1)
    return fail(PPF_ERR_INVALID, "centered must be 0 or 1");
  k.centered = p->centered;
  CUtensorMap map;
  if ((rc = plane_map<T>(&map, in, g, m))) return rc;
  int* st = status_ptr();
  if (!st) return fail(PPF_ERR_CUDA, "status word unavailable");
  dim3 gd((g.n[2] + m.TX - 1) / m.TX, (g.n[1] + m.TY - 1) / m.TY, (g.n[0] + m.ZC - 1) / m.ZC);
  const bool pdl = tiling && tiling->pdl;
  if (quant) {
    auto kern = cahn_hilliard_kernel<T, true>;
    PPF_TRY_CUDA(allow_smem(kern, smem));
    m.ZC = zchunk_of(tiling, g);
    gd.z = (unsigned)((g.n[0] + m.ZC - 1) / m.ZC);
    PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream, pdl,
                        map, k, g, bc, in, out, mass, (int*)status, m, slot_elems, st));
  } else {
    auto kern = cahn_hilliard_kernel<T, false>;
    PPF_TRY_CUDA(allow_smem(kern, smem));
    m.ZC = zchunk_of(tiling, g);
    gd.z = (unsigned)((g.n[0] + m.ZC - 1) / m.ZC);
    PPF_TRY_CUDA(launch(kern, gd, dim3(32, kThreads / 32), smem, (cudaStream_t)stream, pdl,
                        map, k, g, bc, in, out, mass, (int*)status, m, slot_elems, st));
  }
  return PPF_OK;
}

}  // namespace

int32_t diffusion3d_f32(const PpfDiffusionParams* p, const PpfGrid* g, const PpfBoundary* b,
                        const float* in, float* out, const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  return run_march7<float>(Diffusion7<float>{(float)(p->dt * p->D / (p->dx * p->dx))}, p->dx, g,
                           b, in, out, t, s);
}
int32_t diffusion3d_f64(const PpfDiffusionParams* p, const PpfGrid* g, const PpfBoundary* b,
                        const double* in, double* out, const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  return run_march7<double>(Diffusion7<double>{p->dt * p->D / (p->dx * p->dx)}, p->dx, g, b, in,
                            out, t, s);
}
int32_t allen_cahn3d_f32(const PpfAllenCahnParams* p, const PpfGrid* g, const PpfBoundary* b,
                         const float* in, float* out, const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  AllenCahn7<float> op{(float)(p->dt * p->M * p->epsilon * p->epsilon / (p->dx * p->dx)),
                       (float)(p->dt * p->M * 16.0 * p->W)};
  return run_march7<float>(op, p->dx, g, b, in, out, t, s);
}
int32_t allen_cahn3d_f64(const PpfAllenCahnParams* p, const PpfGrid* g, const PpfBoundary* b,
                         const double* in, double* out, const PpfTiling* t, void* s) {
  clear_error();
  if (!p || !(p->dx > 0)) return fail(PPF_ERR_INVALID, "bad params");
  AllenCahn7<double> op{p->dt * p->M * p->epsilon * p->epsilon / (p->dx * p->dx),
                        p->dt * p->M * 16.0 * p->W};
  return run_march7<double>(op, p->dx, g, b, in, out, t, s);
}

}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_cahn_hilliard_step_f32(const PpfCahnHilliardParams* p, const PpfGrid* g,
                                   const PpfBoundary* bc, const float* in, float* out,
                                   double* mass_accum, int32_t* status, const PpfTiling* tiling,
                                   void* stream) {
  return cahn_hilliard<float>(p, g, bc, in, out, mass_accum, status, tiling, stream);
}
int32_t ppf_cahn_hilliard_step_f64(const PpfCahnHilliardParams* p, const PpfGrid* g,
                                   const PpfBoundary* bc, const double* in, double* out,
                                   double* mass_accum, int32_t* status, const PpfTiling* tiling,
                                   void* stream) {
  return cahn_hilliard<double>(p, g, bc, in, out, mass_accum, status, tiling, stream);
}

}  // extern "C"
