// 2-D Diffusion and Allen-Cahn explicit steps, one or several per pass.
//
// Kernels: stencil2d_lean_kernel (one step, warp strips of 16-byte
// vectors, the default), stencil2d_march_kernel (depth 2..8 steps per HBM
// pass: warps march down column windows fed by TMA, a pipeline of one
// register stage per step) and stencil2d_tb_kernel (depth steps on a
// TY x TX shared-memory tile with a halo of `depth` cells, used when a tile
// shape is asked for). Every kernel reads each cell once and writes it once
// per pass, applying the ghost rule at load time.
//
// Reference: engine_ExplicitDiffusion (Engines/Diffusion.py:198-208) and
// engine_CahnAllenExplicit (Engines/CahnAllen.py:128-135), with Field.laplacian
// (field.py:60-67) as the 5-point stencil.
#include "ppf_common.cuh"
#include "ppf_tma.cuh"

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

// ------------------------------------------------------------ marching
// Temporal blocking by marching (depth K = 2..8 steps per HBM pass). A warp
// owns a window of 32 V columns (V cells of one 16-byte vector per lane) and
// a segment of `seg` output rows. It reads the segment's rows plus K halo
// rows above and below once, top to bottom, and pushes each row through a
// pipeline of K stages held in registers: stage k keeps two rows of step
// k-1 and, when the next row of step k-1 arrives, emits one row of step k
// (west / east neighbours by shuffles). Only stage K's rows go back to
// memory, so HBM sees one read and one write per cell per K steps, plus the
// 2K halo rows per segment. The window's outer KA = K rounded up to V
// columns per side are halo (lost one column per step); lanes KA/V ..
// 31 - KA/V own the output columns, so neighbouring windows overlap by 2 KA.
//
// Rows arrive through a per-warp ring of kMSlots shared-memory slots of
// kMRows rows each, filled by TMA tensor loads (cp.async.bulk.tensor.2d,
// one lane, completion on the slot's mbarrier; every wait bounded) while
// earlier slots are consumed. Blocks of rows that reach outside the grid
// (the grid's first and last rows, windows over the left or right edge) are
// filled by the warp itself with the boundary rule instead; the ghost cells
// they hold then evolve with the stencil like the cells they copy (periodic
// wrap, no-flux mirror: the neighbour sum ((w + e) + (n + s)) is symmetric,
// so a mirrored cell stays bit-identical to its image), and Dirichlet
// ghosts keep their value at every step.
constexpr int kMWarps = 4;
constexpr int kMRows = 4;
constexpr int kMSlots = 4;

// A block of kMRows rows of a window filled by the warp itself with the
// boundary rule (edges of the grid); kept out of line, off the hot path.
template <typename T, int V>
__device__ __noinline__ void march_fill(T* dst, const T* __restrict__ in, const Geo* g,
                                        const Bc<T>* bc, int r0, int xl, int lane) {
  for (int r = 0; r < kMRows; ++r)
    for (int e = 0; e < V; ++e)
      dst[r * 32 * V + lane * V + e] = fetch<T, 2>(in, *g, *bc, 0, r0 + r, xl + e);
  __syncwarp();
}

// Resident CTAs per SM asked of the register allocator: the pipeline holds
// 2 K V values per lane, so deeper pipelines get fewer CTAs (shared memory
// allows seven).
template <typename T, int K>
struct MarchMinBlocks {
  static constexpr int regs = 8 * K + 64;  // pipeline (2 K vectors of 16 bytes) + the rest
  static constexpr int fit = 65536 / (32 * kMWarps * regs);
  static constexpr int value = fit > 7 ? 7 : fit;
};

template <typename T, typename Op, int K>
__global__ void __launch_bounds__(32 * kMWarps, (MarchMinBlocks<T, K>::value))
    stencil2d_march_kernel(const __grid_constant__ CUtensorMap map, Op op,
                           const __grid_constant__ Geo g, const __grid_constant__ Bc<T> bc,
                           const T* __restrict__ in, T* __restrict__ out, int ow, int seg,
                           int nstrips, int* __restrict__ status) {
  constexpr int V = Vec16<T>::n;
  using VT = typename Vec16<T>::type;
  constexpr int WW = 32 * V;                    // window columns
  constexpr int KA = (K + V - 1) / V * V;       // halo columns per side
  constexpr int SLOT = kMRows * WW;             // elements per slot
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[kMWarps][kMSlots];
  const int lane = threadIdx.x, wid = threadIdx.y;
  T* ring = reinterpret_cast<T*>(smem_raw) + (size_t)wid * kMSlots * SLOT;
  uint64_t* bar = bars[wid];
  if (lane == 0) {
    for (int i = 0; i < kMSlots; ++i) mbar_init(&bar[i], 1);
    mbar_init_fence();
  }
  __syncwarp();
  pdl_wait();
  pdl_launch_next();
  const int strip = blockIdx.x * kMWarps + wid;
  if (strip >= nstrips) return;  // whole warp; no block-wide barrier follows
  const int ny = g.n[0], nx = g.n[1];
  const int xs = strip * ow - KA;
  const int y0 = blockIdx.y * seg;
  const int y1 = min(y0 + seg, ny);
  const int ylo = y0 - K, yhi = y1 - 1 + K;  // rows read
  const int nb = (yhi - ylo + kMRows) / kMRows;
  const bool xin = xs >= 0 && xs + WW <= nx;
  const int xl = xs + lane * V;  // this lane's first column

  // Dirichlet ghosts along x (edge windows only): those columns never change
  uint32_t fix_x = 0;
#pragma unroll
  for (int e = 0; e < V; ++e)
    if (bc.type[1] == PPF_BC_DIRCHLET && (unsigned)(xl + e) >= (unsigned)nx) fix_x |= 1u << e;
  const bool fix_y = bc.type[0] == PPF_BC_DIRCHLET;

  // blocks whose rows lie in the grid come by TMA (a window over the left
  // or right edge included: the columns outside the grid arrive zero-filled
  // and are rewritten below); the few blocks of rows outside the grid are
  // filled by the warp
  auto tma_block = [&](int b) {
    const int r0 = ylo + b * kMRows;
    return r0 >= 0 && r0 + kMRows <= ny;
  };
  auto issue = [&](int b) {
    const int slot = b % kMSlots;
    T* dst = ring + slot * SLOT;
    const int r0 = ylo + b * kMRows;
    if (tma_block(b)) {
      if (lane == 0) {
        fence_proxy_async();
        mbar_expect_tx(&bar[slot], SLOT * (uint32_t)sizeof(T));
        tma_load_2d(dst, &map, xs, r0, &bar[slot]);
      }
    } else {
      march_fill<T, V>(dst, in, &g, &bc, r0, xl, lane);
    }
  };

  // pipeline state: stage k keeps rows (r - 1, r) of step k - 1
  T wa[K][V], wb[K][V];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int e = 0; e < V; ++e) wa[k][e] = wb[k][e] = T(0);
  const bool owner = lane >= KA / V && lane <= 31 - KA / V;

  for (int b = 0; b < min(kMSlots, nb); ++b) issue(b);
  uint32_t phase = 0;
  for (int b = 0; b < nb; ++b) {
    const int slot = b % kMSlots;
    if (tma_block(b)) {
      if (!mbar_wait_poll(&bar[slot], (phase >> slot) & 1u)) {
        if (lane == 0) {
          atomicOr(status, PPF_STATUS_TIMEOUT);
          // let every load still in flight land before the warp leaves
          // (blocks b .. b + kMSlots - 1 occupy distinct slots, none consumed)
          for (int q = b; q < min(b + kMSlots, nb); ++q)
            if (tma_block(q)) mbar_wait(&bar[q % kMSlots], (phase >> (q % kMSlots)) & 1u);
        }
        __syncwarp();
        return;
      }
      phase ^= 1u << slot;
      if (!xin) {  // the window's cells outside the grid, by the boundary rule
        T* dst = ring + slot * SLOT;
        const int r0 = ylo + b * kMRows;
#pragma unroll
        for (int e = 0; e < V; ++e)
          if ((unsigned)(xl + e) >= (unsigned)nx)
            for (int r = 0; r < kMRows; ++r)
              dst[r * WW + lane * V + e] = fetch<T, 2>(in, g, bc, 0, r0 + r, xl + e);
        __syncwarp();
      }
    }
    const T* src = ring + slot * SLOT;
    // two rows per iteration: the pipeline registers rotate without copies
#pragma unroll 2
    for (int r = 0; r < kMRows; ++r) {
      const int y = ylo + b * kMRows + r;  // row of step 0 entering the pipeline
      // (rows past yhi only feed outputs below the segment, never stored)
      T cur[V];
      {
        const VT v = *reinterpret_cast<const VT*>(src + r * WW + lane * V);
        const T* pv = reinterpret_cast<const T*>(&v);
#pragma unroll
        for (int e = 0; e < V; ++e) cur[e] = pv[e];
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        // stage k + 1: rows y - k - 2 (wa), y - k - 1 (wb), y - k (cur) of
        // step k give row y - k - 1 of step k + 1
        const int row = y - k - 1;
        T nxt[V];
        const T wl = __shfl_up_sync(0xffffffffu, wb[k][V - 1], 1);
        const T er = __shfl_down_sync(0xffffffffu, wb[k][0], 1);
#pragma unroll
        for (int e = 0; e < V; ++e) {
          const T w = e == 0 ? wl : wb[k][e - 1];
          const T ea = e == V - 1 ? er : wb[k][e + 1];
          nxt[e] = op(wb[k][e], w, ea, wa[k][e], cur[e]);
        }
        if (fix_x) {
#pragma unroll
          for (int e = 0; e < V; ++e)
            if (fix_x & (1u << e)) nxt[e] = wb[k][e];
        }
        if (fix_y && (unsigned)row >= (unsigned)ny) {
#pragma unroll
          for (int e = 0; e < V; ++e) nxt[e] = wb[k][e];
        }
#pragma unroll
        for (int e = 0; e < V; ++e) {
          wa[k][e] = wb[k][e];
          wb[k][e] = cur[e];
          cur[e] = nxt[e];
        }
      }
      // cur: row y - K of step K
      const int row = y - K;
      if (owner && row >= y0 && row < y1) {
        T* o = out + (int64_t)row * g.pitch + xl;
        if (xl + V <= nx) {
          VT v;
          T* pv = reinterpret_cast<T*>(&v);
#pragma unroll
          for (int e = 0; e < V; ++e) pv[e] = cur[e];
          *reinterpret_cast<VT*>(o) = v;
        } else {
#pragma unroll
          for (int e = 0; e < V; ++e)
            if (xl + e < nx) o[e] = cur[e];
        }
      }
    }
    // every lane's reads of the slot are ordered before the TMA that refills it
    fence_proxy_async();
    __syncwarp();
    if (b + kMSlots < nb) issue(b + kMSlots);
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

// Segment rows per warp: short enough for about four waves of CTAs, so
// that CTAs that run slower (their rows sit in the other die's memory, or
// they hold the grid's edges) are balanced by the scheduler; one wave of long
// segments measured 40 % slower. Between 16K rows (the 2K halo rows re-read
// per segment cost 12 %) and 64K rows.
inline int march_segment(int ny, int nstrips, int K, long resident) {
  const long cols = (nstrips + kMWarps - 1) / kMWarps;
  long seg = ((long)ny * cols + 4 * resident - 1) / (4 * resident);
  if (seg < 16L * K) seg = 16L * K;
  if (seg > 64L * K) seg = 64L * K;
  seg = (seg + kMRows - 1) / kMRows * kMRows;
  const long full = (ny + kMRows - 1) / kMRows * kMRows;
  return (int)(seg < full ? seg : full);
}

template <typename T, typename Op, int K>
int32_t launch_march(const CUtensorMap& map, Op op, const Geo& g, const Bc<T>& bc, const T* in,
                     T* out, int ow, int seg_req, int nstrips, int* st, bool pdl,
                     cudaStream_t s) {
  constexpr int WW = 32 * Vec16<T>::n;
  const size_t smem = (size_t)kMWarps * kMSlots * kMRows * WW * sizeof(T);
  auto kern = stencil2d_march_kernel<T, Op, K>;
  PPF_TRY_CUDA(allow_smem(kern, smem));
  int seg = seg_req;
  if (seg <= 0) {
    int dev = 0, sms = 0, per_sm = 0;
    PPF_TRY_CUDA(cudaGetDevice(&dev));
    PPF_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PPF_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kMWarps,
                                                               smem));
    seg = march_segment(g.n[0], nstrips, K, (long)sms * (per_sm < 1 ? 1 : per_sm));
  }
  const long gy = (g.n[0] + seg - 1) / seg;
  if (gy > 65535) return fail(PPF_ERR_INVALID, "too many row segments");
  dim3 grid_dim((nstrips + kMWarps - 1) / kMWarps, (unsigned)gy);
  PPF_TRY_CUDA(launch(kern, grid_dim, dim3(32, kMWarps), smem, s, pdl, map, op, g, bc, in, out,
                      ow, seg, nstrips, st));
  return PPF_OK;
}

template <typename T, typename Op>
int32_t run_march(Op op, const Geo& g, const Bc<T>& bc, const T* in, T* out, int K, int seg_req,
                  bool pdl, cudaStream_t s) {
  constexpr int V = Vec16<T>::n;
  constexpr int WW = 32 * V;
  if (((uintptr_t)in) % 16 || ((uintptr_t)out) % 16 || (g.pitch * sizeof(T)) % 16)
    return fail(PPF_ERR_INVALID, "temporal blocking needs 16-byte aligned rows");
  const int KA = (K + V - 1) / V * V;
  const int ow = WW - 2 * KA;
  const int nstrips = (g.n[1] + ow - 1) / ow;
  int seg = seg_req > 0 ? (seg_req + kMRows - 1) / kMRows * kMRows : 0;
  CUtensorMap map;
  const uint64_t dims[2] = {(uint64_t)g.n[1], (uint64_t)g.n[0]};
  const uint64_t strides[1] = {(uint64_t)g.pitch * sizeof(T)};
  const uint32_t box[2] = {(uint32_t)WW, (uint32_t)kMRows};
  int32_t rc = tensor_map(&map, in, (int)sizeof(T), 2, dims, strides, box);
  if (rc) return rc;
  int* st = status_ptr();
  if (!st) return fail(PPF_ERR_CUDA, "status word unavailable");
  switch (K) {
    case 2: return launch_march<T, Op, 2>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    case 3: return launch_march<T, Op, 3>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    case 4: return launch_march<T, Op, 4>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    case 5: return launch_march<T, Op, 5>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    case 6: return launch_march<T, Op, 6>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    case 7: return launch_march<T, Op, 7>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    case 8: return launch_march<T, Op, 8>(map, op, g, bc, in, out, ow, seg, nstrips, st, pdl, s);
    default: return fail(PPF_ERR_INVALID, "depth=%d not in [2, 8]", K);
  }
}

template <typename T, typename Op>
int32_t run2d(Op op, double dx, const PpfGrid* grid, const PpfBoundary* b,
              const T* in, T* out, const PpfTiling* tiling, void* stream) {
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (in == out) return fail(PPF_ERR_INVALID, "in and out must differ");
  const int depth = tiling && tiling->depth ? tiling->depth : 1;
  if (depth > 1 && !(tiling && tiling->tile_x)) {
    if (depth > 8) return fail(PPF_ERR_INVALID, "depth=%d not in [1, 8]", depth);
    Bc<T> bcm;
    if ((rc = make_bc<T>(b, g, dx, 1, depth, &bcm))) return rc;
    return run_march<T, Op>(op, g, bcm, in, out, depth, tiling->tile_y, tiling->pdl != 0,
                            (cudaStream_t)stream);
  }
  Tile2d t;
  if ((rc = plan_tile2d<T>(tiling, &t))) return rc;
  Bc<T> bc;
  if ((rc = make_bc<T>(b, g, dx, 1, t.k, &bc))) return rc;
  const int vec_ok = (((uintptr_t)in) % 16 == 0) && (((uintptr_t)out) % 16 == 0) &&
                     ((g.pitch * sizeof(T)) % 16 == 0);
  const bool pdl = tiling && tiling->pdl;
  if (t.k == 1 && !(tiling && tiling->tile_x)) {
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
