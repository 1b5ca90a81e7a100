// Kernels of the learned surrogate (a convolutional encoder-decoder that
// advances the Warren1995 (phi, c) state by k stencil steps): a BF16
// tensor-core GEMM with FP32 accumulation whose operand loaders and result
// storers implement the patchify / unpatchify implicit-GEMM convolutions and
// the 1x1 convolutions (forward, data gradient, weight gradient), plus
// depthwise 3x3 convolution, bias, GELU, loss and Adam kernels.
//
// Activations are channels-last: token t = (sample, row, col) of the patch
// grid, channel n contiguous. Weights of a 1x1 / patch convolution are
// W[out][in] (bf16 copy for the GEMM, fp32 master for Adam).
//
// Tensor-core path: mma.sync.m16n8k16 (bf16 x bf16 -> f32). A 64x64 output
// tile per CTA of 4 warps (32x32 each), k in steps of 32 staged in shared
// memory (A row-major, B stored transposed so every fragment register is one
// 32-bit shared load).
#include <cuda_bf16.h>
#include <math.h>

#include <type_traits>

#include "ppf_common.cuh"
#include "ppf_tma.cuh"

namespace ppf {
namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int kGemmThreads = 128;
constexpr int kPad = 8;  // shared row padding (bf16 elements)

// ---------------------------------------------------------------- loaders
// A(m, k) and B(k, n) element accessors (return float; converted to bf16).
struct StridedBf16 {  // element (i, j) = x[i * si + j * sj]
  const __nv_bfloat16* x;
  long long si, sj;
};

// Patch gather of a 2-channel state field stack: rows are tokens
// (b, ty, tx), columns are (ch, py, px) of the P x P patch; fields are fp32
// [b][ch][H][pitch] and are normalised by `scale[ch]` on the fly.
struct PatchGather {
  const float* f;
  int P, H, W, pitch, gh, gw;  // image H x W, patch grid gh x gw
  float o0, s0, o1, s1;        // input normalisation (v - o) * s per channel
  __device__ float operator()(long long t, long long k) const {
    const int per = gh * gw;
    const int b = (int)(t / per);
    const int r = (int)(t - (long long)b * per);
    const int ty = r / gw, tx = r - ty * gw;
    const int ch = (int)(k / (P * P));
    const int q = (int)(k - (long long)ch * P * P);
    const int py = q / P, px = q - py * P;
    const float v = f[(((long long)b * 2 + ch) * H + ty * P + py) * pitch + tx * P + px];
    return ch == 0 ? (v - o0) * s0 : (v - o1) * s1;
  }
};

// The same gather seen as B(k = token, n = (ch, py, px)) for weight grads.
struct PatchGatherT {
  PatchGather g;
  __device__ float operator()(long long k, long long n) const { return g(k, n); }
};

// ---------------------------------------------------------------- storers
// C(m, n) epilogues. All receive the fp32 accumulator.
struct StoreF32 {  // y[m * ld + n] (= or +=) acc + bias[n]
  float* y;
  const float* bias;
  long long ld;
  int accumulate;
  __device__ void operator()(long long m, long long n, float v) const {
    if (bias) v += bias[n];
    float* p = y + m * ld + n;
    if (accumulate) *p += v;
    else *p = v;
  }
};

struct StoreBf16Pair {  // fp32 and bf16 copies of acc + bias (no activation)
  float* y;
  __nv_bfloat16* yb;
  const float* bias;
  long long ld;
  __device__ void operator()(long long m, long long n, float v) const {
    if (bias) v += bias[n];
    y[m * ld + n] = v;
    yb[m * ld + n] = __float2bfloat16(v);
  }
};

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

struct StoreGelu {  // pre = acc + bias (fp32), act = gelu(pre) (bf16)
  float* pre;
  __nv_bfloat16* act;
  const float* bias;
  long long ld;
  __device__ void operator()(long long m, long long n, float v) const {
    v += bias[n];
    pre[m * ld + n] = v;
    act[m * ld + n] = __float2bfloat16(gelu(v));
  }
};

struct StoreGeluGrad {  // d_pre = acc * gelu'(pre), bf16
  const float* pre;
  __nv_bfloat16* dpre;
  long long ld;
  __device__ void operator()(long long m, long long n, float v) const {
    dpre[m * ld + n] = __float2bfloat16(v * gelu_grad(pre[m * ld + n]));
  }
};

struct StoreResidual {  // y += acc + bias, keep a bf16 copy of the new y
  float* y;
  __nv_bfloat16* yb;
  const float* bias;
  long long ld;
  __device__ void operator()(long long m, long long n, float v) const {
    const float r = y[m * ld + n] + v + bias[n];
    y[m * ld + n] = r;
    yb[m * ld + n] = __float2bfloat16(r);
  }
};

struct StoreAtomic {  // y[m * ld + n] += acc (split-k weight gradients)
  float* y;
  long long ld;
  __device__ void operator()(long long m, long long n, float v) const {
    atomicAdd(y + m * ld + n, v);
  }
};

// ---------------------------------------------------------------- GEMM
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Shared tile fill (64 rows x BK columns): S[r][c] = operand element
// (row r0 + r, column c0 + c); zero outside rows < R, columns < ce.
// Generic loaders: consecutive threads take consecutive loader columns
// (the patch gather's pixel index), i.e. tile columns for A, rows for B.
template <typename LD, bool kTransposed>
__device__ __forceinline__ void fill_tile(__nv_bfloat16 (*S)[BK + kPad], const LD& ld, long long r0,
                                          long long R, long long c0, long long ce, int tid) {
  for (int i = tid; i < 64 * BK; i += kGemmThreads) {
    const int r = kTransposed ? i % 64 : i / BK;
    const int c = kTransposed ? i / 64 : i % BK;
    const long long gr = r0 + r, gc = c0 + c;
    float v = 0.f;
    if (gr < R && gc < ce) v = kTransposed ? ld(gc, gr) : ld(gr, gc);
    S[r][c] = __float2bfloat16(v);
  }
}

// Strided bf16 operands: element (r, c) = x[r * rs + c * cs]. Unit column
// stride: 16-byte vector loads where aligned; unit row stride: consecutive
// threads take consecutive rows (coalesced), otherwise scalar.
__device__ __forceinline__ void fill_strided(__nv_bfloat16 (*S)[BK + kPad],
                                             const __nv_bfloat16* __restrict__ x, long long rs,
                                             long long cs, long long r0, long long R, long long c0,
                                             long long ce, int tid) {
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  if (cs == 1) {
    const bool vec = (rs & 7) == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
    for (int i = tid; i < 64 * (BK / 8); i += kGemmThreads) {
      const int r = i / (BK / 8), c = (i - r * (BK / 8)) * 8;
      const long long gr = r0 + r, gc = c0 + c;
      if (vec && gr < R && gc + 8 <= ce) {
        *reinterpret_cast<uint4*>(&S[r][c]) = *reinterpret_cast<const uint4*>(x + gr * rs + gc);
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) S[r][c + q] = (gr < R && gc + q < ce) ? x[gr * rs + gc + q] : zero;
      }
    }
  } else {
    for (int i = tid; i < 64 * BK; i += kGemmThreads) {
      const int c = i / 64, r = i - c * 64;
      const long long gr = r0 + r, gc = c0 + c;
      S[r][c] = (gr < R && gc < ce) ? x[gr * rs + gc * cs] : zero;
    }
  }
}

template <typename LA>
__device__ __forceinline__ void fill_a(__nv_bfloat16 (*S)[BK + kPad], const LA& la, long long m0,
                                       long long M, long long k0, long long ke, int tid) {
  fill_tile<LA, false>(S, la, m0, M, k0, ke, tid);
}
__device__ __forceinline__ void fill_a(__nv_bfloat16 (*S)[BK + kPad], const StridedBf16& la,
                                       long long m0, long long M, long long k0, long long ke,
                                       int tid) {
  fill_strided(S, la.x + m0 * la.si + k0 * la.sj, la.si, la.sj, 0, M - m0, 0, ke - k0, tid);
}
// B tiles are stored transposed: S[n - n0][k - k0] = B(k, n).
template <typename LB>
__device__ __forceinline__ void fill_b(__nv_bfloat16 (*S)[BK + kPad], const LB& lb, long long n0,
                                       long long N, long long k0, long long ke, int tid) {
  fill_tile<LB, true>(S, lb, n0, N, k0, ke, tid);
}
__device__ __forceinline__ void fill_b(__nv_bfloat16 (*S)[BK + kPad], const StridedBf16& lb,
                                       long long n0, long long N, long long k0, long long ke,
                                       int tid) {
  fill_strided(S, lb.x + k0 * lb.si + n0 * lb.sj, lb.sj, lb.si, 0, N - n0, 0, ke - k0, tid);
}

// Patch gather, 4 consecutive patch columns (px .. px + 3 of one patch row,
// P a multiple of 4) per 16-byte load: (token t, column k) -> fields
// offset; the columns of a 4-group share channel and patch row.
__device__ __forceinline__ long long patch_offset(const PatchGather& p, long long t, int k) {
  const int per = p.gh * p.gw;
  const int b = (int)(t / per);
  const int r = (int)(t - (long long)b * per);
  const int ty = r / p.gw, tx = r - ty * p.gw;
  const int ch = k / (p.P * p.P);
  const int q = k - ch * p.P * p.P;
  const int py = q / p.P, px = q - py * p.P;
  return (((long long)b * 2 + ch) * p.H + ty * p.P + py) * p.pitch + tx * p.P + px;
}

__device__ __forceinline__ void fill_a(__nv_bfloat16 (*S)[BK + kPad], const PatchGather& la,
                                       long long m0, long long M, long long k0, long long ke,
                                       int tid) {
  if ((la.P & 3) || (la.pitch & 3) || (reinterpret_cast<uintptr_t>(la.f) & 15)) {
    fill_tile<PatchGather, false>(S, la, m0, M, k0, ke, tid);
    return;
  }
  for (int i = tid; i < 64 * (BK / 4); i += kGemmThreads) {
    const int r = i / (BK / 4), c = (i - r * (BK / 4)) * 4;
    const long long m = m0 + r, k = k0 + c;
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (m < M && k + 4 <= ke) {
      const float4 x = *reinterpret_cast<const float4*>(la.f + patch_offset(la, m, (int)k));
      const bool c0 = k < (long long)la.P * la.P;  // channel 0 (the group shares it)
      const float o = c0 ? la.o0 : la.o1, sc = c0 ? la.s0 : la.s1;
      v[0] = (x.x - o) * sc;
      v[1] = (x.y - o) * sc;
      v[2] = (x.z - o) * sc;
      v[3] = (x.w - o) * sc;
    } else if (m < M) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (k + q < ke) v[q] = la(m, k + q);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) S[r][c + q] = __float2bfloat16(v[q]);
  }
}

// B(k = token, n = patch column) of the patch weight gradient: 4
// consecutive n per load, stored transposed (S[n][k]).
__device__ __forceinline__ void fill_b(__nv_bfloat16 (*S)[BK + kPad], const PatchGatherT& lb,
                                       long long n0, long long N, long long k0, long long ke,
                                       int tid) {
  const PatchGather& g = lb.g;
  if ((g.P & 3) || (g.pitch & 3) || (reinterpret_cast<uintptr_t>(g.f) & 15)) {
    fill_tile<PatchGatherT, true>(S, lb, n0, N, k0, ke, tid);
    return;
  }
  for (int i = tid; i < (64 / 4) * BK; i += kGemmThreads) {
    const int c = i / (64 / 4), r = (i - c * (64 / 4)) * 4;  // token column c, n rows r..r+3
    const long long k = k0 + c, n = n0 + r;
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (k < ke && n + 4 <= N) {
      const float4 x = *reinterpret_cast<const float4*>(g.f + patch_offset(g, k, (int)n));
      const bool c0 = n < (long long)g.P * g.P;
      const float o = c0 ? g.o0 : g.o1, sc = c0 ? g.s0 : g.s1;
      v[0] = (x.x - o) * sc;
      v[1] = (x.y - o) * sc;
      v[2] = (x.z - o) * sc;
      v[3] = (x.w - o) * sc;
    } else if (k < ke) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (n + q < N) v[q] = g(k, n + q);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) S[r + q][c] = __float2bfloat16(v[q]);
  }
}

// C(M x N) = sum over k in [k0, k1) of A(m, k) B(k, n); blockIdx.z splits k.
template <typename LA, typename LB, typename ST>
__global__ void __launch_bounds__(kGemmThreads)
    gemm_kernel(LA la, LB lb, ST st, long long M, long long N, long long K, long long kchunk) {
  __shared__ __align__(16) __nv_bfloat16 As[BM][BK + kPad];
  __shared__ __align__(16) __nv_bfloat16 Bt[BN][BK + kPad];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long m0 = (long long)blockIdx.y * BM, n0 = (long long)blockIdx.x * BN;
  const long long kb = (long long)blockIdx.z * kchunk;
  const long long ke = kb + kchunk < K ? kb + kchunk : K;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

  pdl_wait();
  for (long long k0 = kb; k0 < ke; k0 += BK) {
    fill_a(As, la, m0, M, k0, ke, tid);
    fill_b(Bt, lb, n0, N, k0, ke, tid);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t a[2][4], b[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + g;
        a[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t]);
        a[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t]);
        a[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t + 8]);
        a[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + j * 8 + g;
        b[j][0] = *reinterpret_cast<const uint32_t*>(&Bt[c][kk + 2 * t]);
        b[j][1] = *reinterpret_cast<const uint32_t*>(&Bt[c][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const long long m = m0 + wm + i * 16 + g + (r >= 2 ? 8 : 0);
        const long long n = n0 + wn + j * 8 + 2 * t + (r & 1);
        if (m < M && n < N) st(m, n, acc[i][j][r]);
      }
}

// ---------------------------------------------------------------- tcgen05
// The tcgen05 path is on by default for GEMMs of at least kTcMinRows rows
// (the training batches: 8192 tokens x N 384 x K 192 runs at 74 TFLOP/s vs
// 54 on mma.sync, 65536 tokens at 132 vs 86); below that (the 1024-token
// prediction) its few 128 x 128 tiles leave most SMs idle and mma.sync's
// 64 x 64 tiles win. ppf_sg_set_tensor_path(0) selects mma.sync everywhere.
int g_tc_enabled = 1;
constexpr long long kTcMinRows = 4096;
bool tc_enabled() { return g_tc_enabled != 0; }

// 5th-generation tensor-core GEMM for the GEMMs whose operands are both
// K-contiguous bf16 (A[m][k], B stored as [n][k]): the forward 1x1
// convolutions and the output head. One CTA (4 warps) owns a 128 x 128
// output tile whose FP32 accumulator lives in tensor memory (128 lanes x
// 128 columns, allocated by warp 0); k advances in 64-wide tiles staged in
// shared memory in the K-major 128-byte-swizzled layout (8-row x 128-byte
// atoms, 1024 bytes apart along the rows: row r's 16-byte chunk j of k at
// (r / 8) * 1024 + (r % 8) * 128 + ((j ^ (r % 8)) * 16), see tc_desc and
// tc_load_tile). Two stages: the tile for kt + 1 is
// loaded while the tensor core works on kt. One thread issues
// tcgen05.mma (kind::f16, BF16 x BF16 -> F32, M = 128, N = 128, K = 16 per
// instruction) and tcgen05.commit arrives on the stage's mbarrier; the
// epilogue reads the accumulator with tcgen05.ld (warp w: lanes 32w..32w+31
// = rows) and applies the storer. Every mbarrier wait is bounded; a timeout
// sets PPF_STATUS_TIMEOUT, lets the issued MMAs finish (bounded) and frees
// the tensor memory.
constexpr int TCM = 128, TCN = 128, TCK = 64, kTcThreads = 128;
constexpr int kTcStage = (TCM + TCN) * TCK * 2;  // bytes of one A + B stage
constexpr uint32_t kTcIdesc = (1u << 4)                        // D: F32
                              | (1u << 7) | (1u << 10)         // A, B: BF16, K-major
                              | ((uint32_t)(TCN >> 3) << 17)   // N / 8
                              | ((uint32_t)(TCM >> 4) << 24);  // M / 16

__device__ __forceinline__ uint32_t tc_smem(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// shared-memory matrix descriptor: K-major, 128-byte swizzle (8-row x
// 128-byte atoms, stride byte offset 1024 between atoms along M / N; the
// leading offset is implied by the swizzle), descriptor version 1, the tile
// 1024-byte aligned. Stepping K by 16 elements moves the start by 32 bytes.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = tc_smem(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Pipeline: a producer thread (warp 0) streams the k-tiles of A (128 rows)
// and B (128 columns) into kTcStages shared-memory stages with TMA tensor
// loads (cp.async.bulk.tensor.2d, 128-byte swizzle: the K-major SW128 layout
// the descriptors describe), completing on the stage's `full` mbarrier; an
// MMA thread (warp 1) waits for a stage, issues its four tcgen05.mma (K = 16
// each) into the TMEM accumulator and commits onto the stage's `empty`
// mbarrier, which frees the stage for the producer; a final commit onto
// `done` releases the four warps into the epilogue. With three 32 KB stages
// two CTAs share an SM, so one CTA's epilogue overlaps the other's loads.
// Every wait is bounded; a timeout sets PPF_STATUS_TIMEOUT, the issued MMAs
// and loads are waited for (bounded) and the tensor memory is freed.
constexpr int kTcStages = 3;

__device__ __forceinline__ void tc_tma_load(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(tc_smem(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(tc_smem(bar))
      : "memory");
}

template <typename ST>
__global__ void __launch_bounds__(kTcThreads)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap map_a,
                   const __grid_constant__ CUtensorMap map_b, ST st, long long M, long long N,
                   long long K, int* __restrict__ lib_status) {
  extern __shared__ __align__(1024) uint8_t tc_stage[];
  __shared__ __align__(8) uint64_t full[kTcStages], empty[kTcStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag, consumed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long m0 = (long long)blockIdx.y * TCM, n0 = (long long)blockIdx.x * TCN;
  uint8_t* const base = tc_stage + ((1024 - (tc_smem(tc_stage) & 1023)) & 1023);
  auto sa = [&](int st_) { return base + st_ * kTcStage; };
  auto sb = [&](int st_) { return base + st_ * kTcStage + TCM * TCK * 2; };
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(tc_smem(&tmem_base)), "r"(TCN) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < kTcStages; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&full[i])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&empty[i])) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&done)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    consumed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  pdl_wait();
  pdl_launch_next();
  const int nk = (int)((K + TCK - 1) / TCK);
  constexpr uint32_t kLimit = 1u << 15;
  int issued = 0;
  if (warp == 0 && lane == 0) {  // producer
    for (int kt = 0; kt < nk; ++kt) {
      const int s = kt % kTcStages;
      if (kt >= kTcStages &&
          !tc_wait(&empty[s], (uint32_t)((kt / kTcStages - 1) & 1), kLimit)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      if (*(volatile int*)&abort_flag) break;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   ::"r"(tc_smem(&full[s])), "r"((uint32_t)kTcStage) : "memory");
      tc_tma_load(sa(s), &map_a, kt * TCK, (int)m0, &full[s]);
      tc_tma_load(sb(s), &map_b, kt * TCK, (int)n0, &full[s]);
      issued = kt + 1;
    }
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    int kt = 0;
    for (; kt < nk; ++kt) {
      const int s = kt % kTcStages;
      if (!tc_wait(&full[s], (uint32_t)((kt / kTcStages) & 1), kLimit)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < TCK / 16; ++kk) {
        const uint64_t da = tc_desc(tc_smem(sa(s)) + kk * 32);
        const uint64_t db = tc_desc(tc_smem(sb(s)) + kk * 32);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
            ::"r"(tmem), "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc) : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(tc_smem(&empty[s])) : "memory");
    }
    consumed = kt;
    // completes once every MMA issued above has (also after an abort)
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
        ::"r"(tc_smem(&done)) : "memory");
  }
  bool ok = tc_wait(&done, 0u, kLimit);
  ok = !__syncthreads_or(!ok || abort_flag);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // lane = row of the accumulator; 32 columns per round go through a
    // per-warp 32 x 33 shared tile so that the storer runs with consecutive
    // lanes on consecutive columns (coalesced global writes)
    float* tile = reinterpret_cast<float*>(base) + warp * 32 * 33;
#pragma unroll 1
    for (int c0 = 0; c0 < TCN; c0 += 32) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t r[16];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c0 + 16 * h);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
            "%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) tile[lane * 33 + 16 * h + j] = __uint_as_float(r[j]);
      }
      __syncwarp();
      const long long n = n0 + c0 + lane;
#pragma unroll 4
      for (int rr = 0; rr < 32; ++rr) {
        const long long m = m0 + warp * 32 + rr;
        if (m < M && n < N) st(m, n, tile[rr * 33 + lane]);
      }
      __syncwarp();
    }
  } else {
    if (tid == 0) atomicOr(lib_status, PPF_STATUS_TIMEOUT);
    // the MMAs: `done` completes when they have; the loads issued but not
    // consumed: their stages' `full` phases
    if (tid == 0) tc_wait(&done, 0u, kLimit);
    if (warp == 0 && lane == 0)
      for (int kt = consumed; kt < issued; ++kt)
        tc_wait(&full[kt % kTcStages], (uint32_t)((kt / kTcStages) & 1), kLimit);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCN)
                 : "memory");
}

// Whether the tcgen05 kernel applies: both operands K-contiguous with rows
// on 16-byte boundaries, K a multiple of 8, enough rows to fill the GPU
// with its 128 x 128 tiles.
bool tc_eligible(const StridedBf16& la, const StridedBf16& lb, long long M, long long K) {
  return la.sj == 1 && lb.si == 1 && (la.si & 7) == 0 && (lb.sj & 7) == 0 && (K & 7) == 0 &&
         (reinterpret_cast<uintptr_t>(la.x) & 15) == 0 &&
         (reinterpret_cast<uintptr_t>(lb.x) & 15) == 0 && M >= kTcMinRows;
}

template <typename ST>
int32_t tc_gemm(const StridedBf16& la, const StridedBf16& lb, ST st, long long M, long long N,
                long long K, cudaStream_t s) {
  int* status = status_ptr();
  if (!status) return fail(PPF_ERR_CUDA, "status word unavailable");
  if (M > (1LL << 31) - 1 || N > (1LL << 31) - 1 || K > (1LL << 31) - 1)
    return fail(PPF_ERR_INVALID, "GEMM too large");
  CUtensorMap ma, mb;
  int32_t rc = tensor_map_bf16_sw128(&ma, la.x, (uint64_t)K, (uint64_t)M,
                                     (uint64_t)la.si * 2, TCK, TCM);
  if (rc) return rc;
  if ((rc = tensor_map_bf16_sw128(&mb, lb.x, (uint64_t)K, (uint64_t)N, (uint64_t)lb.sj * 2, TCK,
                                  TCN)))
    return rc;
  const size_t smem = (size_t)kTcStages * kTcStage + 1024;
  auto kern = tc_gemm_kernel<ST>;
  PPF_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)((N + TCN - 1) / TCN), (unsigned)((M + TCM - 1) / TCM));
  if (grid.y > 65535) return fail(PPF_ERR_INVALID, "GEMM too large");
  PPF_TRY_CUDA(launch(kern, grid, dim3(kTcThreads), smem, s, false, ma, mb, st, M, N, K, status));
  return PPF_OK;
}

template <typename LA, typename LB, typename ST>
int32_t gemm(LA la, LB lb, ST st, long long M, long long N, long long K, int splits,
             cudaStream_t s) {
  if (M < 1 || N < 1 || K < 1) return fail(PPF_ERR_INVALID, "empty GEMM");
  if constexpr (std::is_same<LA, StridedBf16>::value && std::is_same<LB, StridedBf16>::value) {
    if (splits <= 1 && tc_enabled() && tc_eligible(la, lb, M, K))
      return tc_gemm(la, lb, st, M, N, K, s);
  }
  if (splits < 1) splits = 1;
  long long kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + BK - 1) / BK * BK;
  const long long nz = (K + kchunk - 1) / kchunk;
  dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM), (unsigned)nz);
  if (grid.y > 65535 || nz > 65535) return fail(PPF_ERR_INVALID, "GEMM too large");
  gemm_kernel<LA, LB, ST><<<grid, kGemmThreads, 0, s>>>(la, lb, st, M, N, K, kchunk);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// ---------------------------------------------------------------- split-k
// Weight gradients are GEMMs over the token axis (k = tokens, thousands),
// split across CTAs. Each split writes its partial tile to a fixed library
// array (16 MiB) with plain stores, and one pass adds the splits into the
// gradient: far fewer memory operations than one atomic per split and
// element. The array is shared by every call, so weight-gradient calls must
// not overlap on the GPU (the network's passes run on one stream).
constexpr long long kSplitkCap = 4LL << 20;  // floats
__device__ float g_splitk[kSplitkCap];

struct StorePartial {  // part[split][m][n] = acc
  float* part;
  long long ld, zstride;
  __device__ void operator()(long long m, long long n, float v) const {
    part[blockIdx.z * zstride + m * ld + n] = v;
  }
};

__global__ void splitk_reduce_kernel(const float* __restrict__ part, int nz, long long mn,
                                     float* __restrict__ y) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < mn;
       i += (long long)gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int z = 0; z < nz; ++z) acc += part[z * mn + i];
    y[i] += acc;
  }
}

// Device address of g_splitk on the current device (per device and
// context, see SymbolCache); nullptr if the lookup failed.
float* splitk_buffer() {
  static SymbolCache cache;
  void* p = nullptr;
  if (symbol_address(g_splitk, cache, &p) != PPF_OK) {
    cudaGetLastError();
    return nullptr;
  }
  return (float*)p;
}

// y[M x N] += A B with k = tokens (about 256 per split).
template <typename LA, typename LB>
int32_t gemm_wgrad(LA la, LB lb, float* y, long long M, long long N, long long K, cudaStream_t s) {
  long long splits = K / 256;
  const long long cap = kSplitkCap / (M * N);
  if (splits > cap) splits = cap;
  if (splits > 1024) splits = 1024;
  float* part = splits > 1 ? splitk_buffer() : nullptr;
  if (splits <= 1 || !part) return gemm(la, lb, StoreF32{y, nullptr, N, 1}, M, N, K, 1, s);
  long long kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + BK - 1) / BK * BK;
  const int nz = (int)((K + kchunk - 1) / kchunk);
  int32_t rc = gemm(la, lb, StorePartial{part, N, M * N}, M, N, K, (int)splits, s);
  if (rc) return rc;
  const long long mn = M * N;
  long long blocks = (mn + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  splitk_reduce_kernel<<<(unsigned)blocks, 256, 0, s>>>(part, nz, mn, y);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// ---------------------------------------------------------------- others
// Depthwise 3x3 convolution over the patch grid (zero padding at each
// sample's edge): h[t, c] = bd[c] + sum w[c][dy][dx] y[(row+dy-1, col+dx-1), c].
__global__ void dwconv_fwd_kernel(const float* __restrict__ y, const float* __restrict__ w,
                                  const float* __restrict__ bd, float* __restrict__ h,
                                  __nv_bfloat16* __restrict__ hb, long long T, int C, int gh,
                                  int gw) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T * C) return;
  const long long t = i / C;
  const int c = (int)(i - t * C);
  const int per = gh * gw;
  const int r = (int)(t % per), row = r / gw, col = r - row * gw;
  float acc = bd[c];
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
      const int rr = row + dy, cc = col + dx;
      if ((unsigned)rr < (unsigned)gh && (unsigned)cc < (unsigned)gw)
        acc += w[c * 9 + (dy + 1) * 3 + (dx + 1)] * y[(t + (long long)dy * gw + dx) * C + c];
    }
  h[i] = acc;
  hb[i] = __float2bfloat16(acc);
}

// dY[t, c] += sum w[c][dy][dx] dh[(row-dy+1, col-dx+1), c]
__global__ void dwconv_bwd_data_kernel(const float* __restrict__ dh, const float* __restrict__ w,
                                       float* __restrict__ dy_out, long long T, int C, int gh,
                                       int gw) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T * C) return;
  const long long t = i / C;
  const int c = (int)(i - t * C);
  const int per = gh * gw;
  const int r = (int)(t % per), row = r / gw, col = r - row * gw;
  float acc = 0.f;
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
      const int rr = row - dy, cc = col - dx;
      if ((unsigned)rr < (unsigned)gh && (unsigned)cc < (unsigned)gw)
        acc += w[c * 9 + (dy + 1) * 3 + (dx + 1)] * dh[(t - (long long)dy * gw - dx) * C + c];
    }
  dy_out[i] += acc;
}

// dW[c][dy][dx] += sum_t dh[t, c] y[t + off, c];  dB[c] += sum_t dh[t, c].
// Thread = channel (consecutive threads read consecutive channels of a
// token: coalesced), CTA = a chunk of tokens; per-thread sums, then one
// atomic per (CTA, channel, tap).
__global__ void dwconv_bwd_weight_kernel(const float* __restrict__ dh, const float* __restrict__ y,
                                         float* __restrict__ dw, float* __restrict__ db,
                                         long long T, int C, int gh, int gw, long long chunk) {
  const int c = blockIdx.y * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const long long t0 = (long long)blockIdx.x * chunk;
  const long long t1 = t0 + chunk < T ? t0 + chunk : T;
  const int per = gh * gw;
  float acc[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = 0.f;
  int r = (int)(t0 % per), row = r / gw, col = r - row * gw;
#pragma unroll 4
  for (long long t = t0; t < t1; ++t) {
    const float d = dh[t * C + c];
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int rr = row + dy, cc = col + dx;
        if ((unsigned)rr < (unsigned)gh && (unsigned)cc < (unsigned)gw)
          acc[(dy + 1) * 3 + (dx + 1)] += d * y[(t + (long long)dy * gw + dx) * C + c];
      }
    acc[9] += d;
    if (++col == gw) {  // next token: (row, col) of the patch grid
      col = 0;
      if (++row == gh) row = 0;
    }
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) atomicAdd(dw + c * 9 + q, acc[q]);
  atomicAdd(db + c, acc[9]);
}

// db[n] += sum_m x[m * ld + n] (bias gradient), one thread per column chunk.
__global__ void colsum_kernel(const float* __restrict__ x, const __nv_bfloat16* __restrict__ xb,
                              float* __restrict__ db, long long M, int N, long long chunk) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const long long m0 = (long long)blockIdx.y * chunk;
  const long long m1 = m0 + chunk < M ? m0 + chunk : M;
  float acc = 0.f;
  for (long long m = m0; m < m1; ++m)
    acc += x ? x[m * N + n] : __bfloat162float(xb[m * N + n]);
  atomicAdd(db + n, acc);
}

// Loss on the network output out[t, (ch, py, px)] against the normalised
// target change: d = out - (new - old) * scale[ch]; loss += d^2 / count;
// grad (bf16) = 2 d / count.
__global__ void mse_kernel(const float* __restrict__ out, const float* __restrict__ f_old,
                           const float* __restrict__ f_new, __nv_bfloat16* __restrict__ grad,
                           double* __restrict__ loss, long long T, int P, int H, int pitch,
                           int gh, int gw, float s0, float s1, float inv_count) {
  const int K = 2 * P * P;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float d = 0.f;
  if (i < T * K) {
    const long long t = i / K;
    const int k = (int)(i - t * K);
    const int per = gh * gw;
    const int b = (int)(t / per), r = (int)(t - (long long)b * per);
    const int ty = r / gw, tx = r - ty * gw;
    const int ch = k / (P * P), q = k - ch * P * P, py = q / P, px = q - py * P;
    const long long o = (((long long)b * 2 + ch) * H + ty * P + py) * pitch + tx * P + px;
    d = out[i] - (f_new[o] - f_old[o]) * (ch == 0 ? s0 : s1);
    grad[i] = __float2bfloat16(2.f * d * inv_count);
  }
  float v = d * d * inv_count;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __shared__ float part[8];  // blockDim.x == 256
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int w = 0; w < 8; ++w) sum += part[w];
    if (sum != 0.0) atomicAdd(loss, sum);  // one atomic per block, not per warp
  }
}

// new = old + out / scale[ch] (the surrogate's k-step prediction), fields
// [b][ch][H][pitch], out [token][(ch, py, px)].
__global__ void apply_kernel(const float* __restrict__ out, const float* __restrict__ f_old,
                             float* __restrict__ f_new, long long T, int P, int H, int pitch,
                             int gh, int gw, float inv_s0, float inv_s1, float lo0, float hi0,
                             float lo1, float hi1) {
  const int K = 2 * P * P;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T * K) return;
  const long long t = i / K;
  const int k = (int)(i - t * K);
  const int per = gh * gw;
  const int b = (int)(t / per), r = (int)(t - (long long)b * per);
  const int ty = r / gw, tx = r - ty * gw;
  const int ch = k / (P * P), q = k - ch * P * P, py = q / P, px = q - py * P;
  const long long o = (((long long)b * 2 + ch) * H + ty * P + py) * pitch + tx * P + px;
  const float v = f_old[o] + out[i] * (ch == 0 ? inv_s0 : inv_s1);
  const float lo = ch == 0 ? lo0 : lo1, hi = ch == 0 ? hi0 : hi1;
  f_new[o] = v < lo ? lo : (v > hi ? hi : v);  // a NaN stays NaN for the check to see
}

// Adam (bias-corrected) on fp32 master weights; refreshes the bf16 copy.
__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ wb,
                            const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, long long n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = v;
  const float upd = (a / c1) / (sqrtf(v / c2) + eps) + wd * w[i];
  const float nw = w[i] - lr * upd;
  w[i] = nw;
  if (wb) wb[i] = __float2bfloat16(nw);
}

__global__ void cast_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y,
                            long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// Window check of a k-step prediction p from state u, given s = one stencil
// step from p. Per sample b (fields [b][ch][H][pitch], phi = channel 0):
//   out[3b]   += sum over phi cells of (k (s - p) - (p - u))^2
//   out[3b+1] += sum over phi cells of p^2
//   out[3b+2] += number of cells where p or s holds a non-finite value
__global__ void residual_kernel(const float* __restrict__ u, const float* __restrict__ p,
                                const float* __restrict__ sp, int H, int W, int pitch, float k,
                                double* __restrict__ out) {
  const int b = blockIdx.y;
  const long long plane = (long long)H * pitch;
  const float* u0 = u + (long long)b * 2 * plane;
  const float* p0 = p + (long long)b * 2 * plane;
  const float* s0 = sp + (long long)b * 2 * plane;
  double num = 0.0, den = 0.0, bad = 0.0;
  const long long n = (long long)H * W;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long row = i / W;
    const long long o = row * pitch + (i - row * W);
    const float pv = p0[o], pc = p0[plane + o], sv = s0[o], sc = s0[plane + o];
    const float r = k * (sv - pv) - (pv - u0[o]);
    num += (double)r * r;
    den += (double)pv * pv;
    bad += (isfinite(pv) && isfinite(pc) && isfinite(sv) && isfinite(sc)) ? 0.0 : 1.0;
  }
  for (int off = 16; off > 0; off >>= 1) {
    num += __shfl_xor_sync(0xffffffffu, num, off);
    den += __shfl_xor_sync(0xffffffffu, den, off);
    bad += __shfl_xor_sync(0xffffffffu, bad, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out + 3 * b, num);
    atomicAdd(out + 3 * b + 1, den);
    if (bad != 0.0) atomicAdd(out + 3 * b + 2, bad);
  }
}

int32_t grid1d(long long n, unsigned* blocks) {
  const long long b = (n + 255) / 256;
  if (b < 1 || b > (1LL << 31) - 1) return fail(PPF_ERR_INVALID, "size out of range");
  *blocks = (unsigned)b;
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

// C[M, N] = A[M, K] B[K, N] with bf16 operands given by element strides
// (A(m, k) = a[m*sam + k*sak], B(k, n) = b[k*sbk + n*sbn]) and fp32 result
// y[m*ldy + n] (= or += when accumulate) + bias[n]. splits > 1 splits k
// over CTAs and requires accumulate (atomic adds).
int32_t ppf_sg_gemm(const void* a, long long sam, long long sak, const void* b, long long sbk,
                    long long sbn, float* y, long long ldy, const float* bias, int32_t accumulate,
                    long long M, long long N, long long K, int32_t splits, void* stream) {
  clear_error();
  if (!a || !b || !y) return fail(PPF_ERR_INVALID, "NULL operand");
  StridedBf16 la{(const __nv_bfloat16*)a, sam, sak};
  StridedBf16 lb{(const __nv_bfloat16*)b, sbk, sbn};
  if (splits > 1) {
    if (!accumulate || bias) return fail(PPF_ERR_INVALID, "split-k needs accumulate, no bias");
    return gemm(la, lb, StoreAtomic{y, ldy}, M, N, K, splits, (cudaStream_t)stream);
  }
  return gemm(la, lb, StoreF32{y, bias, ldy, accumulate}, M, N, K, 1, (cudaStream_t)stream);
}

}  // extern "C"

// Network-level entry points (used by pyphasefield_gb300/surrogate.py);
// PpfSgShape is declared in ppf_gb300.h.
extern "C" {

static int32_t sg_check(const PpfSgShape* s) {
  if (!s) return fail(PPF_ERR_INVALID, "shape is NULL");
  if (s->B < 1 || s->P < 1 || s->H % s->P || s->W % s->P || s->pitch < s->W || s->C < 1 ||
      s->E < 1)
    return fail(PPF_ERR_INVALID, "bad surrogate shape");
  return PPF_OK;
}

// Patch embedding: y = patches(fields) Win^T + b, with fp32 and bf16 copies.
int32_t ppf_sg_patch_fwd(const PpfSgShape* s, const float* fields, const void* w_in_bf16,
                         const float* b_in, float* y, void* y_bf16, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw, K = 2LL * s->P * s->P;
  PatchGather la{fields, s->P, s->H, s->W, s->pitch, gh, gw, s->in_off0, s->in_sc0,
                 s->in_off1, s->in_sc1};
  StridedBf16 lb{(const __nv_bfloat16*)w_in_bf16, 1, K};
  return gemm(la, lb, StoreBf16Pair{y, (__nv_bfloat16*)y_bf16, b_in, s->C}, T, s->C, K, 1,
              (cudaStream_t)stream);
}

// dWin += dy^T patches(fields) (split-k over tokens), db_in += column sums
// of dy.
int32_t ppf_sg_patch_bwd_weight(const PpfSgShape* s, const float* fields, const void* dy_bf16,
                                float* dw_in, float* db_in, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw, K = 2LL * s->P * s->P;
  StridedBf16 la{(const __nv_bfloat16*)dy_bf16, 1, s->C};  // A(m = out ch, k = token)
  PatchGatherT lb{{fields, s->P, s->H, s->W, s->pitch, gh, gw, s->in_off0, s->in_sc0,
                   s->in_off1, s->in_sc1}};
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = gemm_wgrad(la, lb, dw_in, s->C, K, T, st))) return rc;
  dim3 cg((unsigned)((s->C + 127) / 128), (unsigned)((T + 31) / 32));
  colsum_kernel<<<cg, 128, 0, st>>>(nullptr, (const __nv_bfloat16*)dy_bf16, db_in, T, s->C, 32);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// Depthwise conv + pointwise expand + GELU: h = dw(y), pre = h W1^T + b1,
// act = gelu(pre) (bf16).
int32_t ppf_sg_block_fwd(const PpfSgShape* s, const float* y, const float* w_dw, const float* b_dw,
                         float* h, void* h_bf16, const void* w1_bf16, const float* b1, float* pre,
                         void* act_bf16, const void* w2_bf16, const float* b2, float* y_out,
                         void* y_out_bf16, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned blocks;
  if ((rc = grid1d(T * s->C, &blocks))) return rc;
  dwconv_fwd_kernel<<<blocks, 256, 0, st>>>(y, w_dw, b_dw, h, (__nv_bfloat16*)h_bf16, T, s->C,
                                            gh, gw);
  PPF_TRY_CUDA(cudaGetLastError());
  StridedBf16 ha{(const __nv_bfloat16*)h_bf16, s->C, 1};
  StridedBf16 w1{(const __nv_bfloat16*)w1_bf16, 1, s->C};  // B(k=c, n=e) = W1[e][c]
  if ((rc = gemm(ha, w1, StoreGelu{pre, (__nv_bfloat16*)act_bf16, b1, s->E}, T, s->E, s->C, 1,
                 st)))
    return rc;
  StridedBf16 aa{(const __nv_bfloat16*)act_bf16, s->E, 1};
  StridedBf16 w2{(const __nv_bfloat16*)w2_bf16, 1, s->E};  // B(k=e, n=c) = W2[c][e]
  // y_out = y + act W2^T + b2 (y_out may alias y)
  if (y_out != y) PPF_TRY_CUDA(cudaMemcpyAsync(y_out, y, T * s->C * sizeof(float),
                                               cudaMemcpyDeviceToDevice, st));
  return gemm(aa, w2, StoreResidual{y_out, (__nv_bfloat16*)y_out_bf16, b2, s->C}, T, s->C, s->E,
              1, st);
}

// Backward of ppf_sg_block_fwd given dy_out (fp32, also bf16 copy):
// dW2, db2, dW1, db1, dWdw, dbdw accumulate; dy (fp32) = dy_out + dwconv^T(dh).
int32_t ppf_sg_block_bwd(const PpfSgShape* s, const float* y, const void* h_bf16,
                         const float* pre, const void* act_bf16, const void* w1_bf16,
                         const void* w2_bf16, const float* w_dw, const float* dy_out,
                         const void* dy_out_bf16, void* dpre_bf16, float* dh, void* dh_bf16,
                         float* dy, float* dw1, float* db1, float* dw2, float* db2, float* dw_dw,
                         float* db_dw, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw;
  cudaStream_t st = (cudaStream_t)stream;
  // dW2[c][e] += sum_t dy_out[t][c] act[t][e]
  StridedBf16 dyT{(const __nv_bfloat16*)dy_out_bf16, 1, s->C};
  StridedBf16 act{(const __nv_bfloat16*)act_bf16, s->E, 1};
  if ((rc = gemm_wgrad(dyT, act, dw2, s->C, s->E, T, st))) return rc;
  const long long chunk = 32;
  dim3 cg((s->C + 127) / 128, (unsigned)((T + chunk - 1) / chunk));
  colsum_kernel<<<cg, 128, 0, st>>>(dy_out, nullptr, db2, T, s->C, chunk);
  PPF_TRY_CUDA(cudaGetLastError());
  // d_act = dy_out W2 ; d_pre = d_act * gelu'(pre)
  StridedBf16 dyA{(const __nv_bfloat16*)dy_out_bf16, s->C, 1};
  StridedBf16 w2{(const __nv_bfloat16*)w2_bf16, s->E, 1};  // B(k=c, n=e) = W2[c][e]
  if ((rc = gemm(dyA, w2, StoreGeluGrad{pre, (__nv_bfloat16*)dpre_bf16, s->E}, T, s->E, s->C, 1,
                 st)))
    return rc;
  // dW1[e][c] += sum_t dpre[t][e] h[t][c] ; db1
  StridedBf16 dpT{(const __nv_bfloat16*)dpre_bf16, 1, s->E};
  StridedBf16 hh{(const __nv_bfloat16*)h_bf16, s->C, 1};
  if ((rc = gemm_wgrad(dpT, hh, dw1, s->E, s->C, T, st))) return rc;
  dim3 cg1((s->E + 127) / 128, (unsigned)((T + chunk - 1) / chunk));
  colsum_kernel<<<cg1, 128, 0, st>>>(nullptr, (const __nv_bfloat16*)dpre_bf16, db1, T, s->E,
                                     chunk);
  PPF_TRY_CUDA(cudaGetLastError());
  // dh = dpre W1
  StridedBf16 dpA{(const __nv_bfloat16*)dpre_bf16, s->E, 1};
  StridedBf16 w1{(const __nv_bfloat16*)w1_bf16, s->C, 1};  // B(k=e, n=c) = W1[e][c]
  if ((rc = gemm(dpA, w1, StoreBf16Pair{dh, (__nv_bfloat16*)dh_bf16, nullptr, s->C}, T, s->C,
                 s->E, 1, st)))
    return rc;
  // depthwise: weight/bias grads, then dy = dy_out + dwconv^T(dh)
  const long long wchunk = 32;
  dim3 wg((unsigned)((T + wchunk - 1) / wchunk), (unsigned)((s->C + 127) / 128));
  dwconv_bwd_weight_kernel<<<wg, 128, 0, st>>>(dh, y, dw_dw, db_dw, T, s->C, gh, gw, wchunk);
  PPF_TRY_CUDA(cudaGetLastError());
  if (dy != dy_out)
    PPF_TRY_CUDA(cudaMemcpyAsync(dy, dy_out, T * s->C * sizeof(float), cudaMemcpyDeviceToDevice,
                                 st));
  unsigned blocks;
  if ((rc = grid1d(T * s->C, &blocks))) return rc;
  dwconv_bwd_data_kernel<<<blocks, 256, 0, st>>>(dh, w_dw, dy, T, s->C, gh, gw);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// Output head: out = y Wout^T + bout, out [token][2 P P].
int32_t ppf_sg_head_fwd(const PpfSgShape* s, const void* y_bf16, const void* w_out_bf16,
                        const float* b_out, float* out, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw, K = 2LL * s->P * s->P;
  StridedBf16 la{(const __nv_bfloat16*)y_bf16, s->C, 1};
  StridedBf16 lb{(const __nv_bfloat16*)w_out_bf16, 1, s->C};  // B(k=c, n=o) = Wout[o][c]
  return gemm(la, lb, StoreF32{out, b_out, K, 0}, T, K, s->C, 1, (cudaStream_t)stream);
}

// Head backward: dWout += dout^T y, dbout, dy = dout Wout (fp32 and bf16).
int32_t ppf_sg_head_bwd(const PpfSgShape* s, const void* y_bf16, const void* w_out_bf16,
                        const void* dout_bf16, float* dw_out, float* db_out, float* dy,
                        void* dy_bf16, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw, K = 2LL * s->P * s->P;
  cudaStream_t st = (cudaStream_t)stream;
  StridedBf16 doT{(const __nv_bfloat16*)dout_bf16, 1, K};
  StridedBf16 yy{(const __nv_bfloat16*)y_bf16, s->C, 1};
  if ((rc = gemm_wgrad(doT, yy, dw_out, K, s->C, T, st))) return rc;
  dim3 cg((unsigned)((K + 127) / 128), (unsigned)((T + 31) / 32));
  colsum_kernel<<<cg, 128, 0, st>>>(nullptr, (const __nv_bfloat16*)dout_bf16, db_out, T, (int)K,
                                    32);
  PPF_TRY_CUDA(cudaGetLastError());
  StridedBf16 doA{(const __nv_bfloat16*)dout_bf16, K, 1};
  StridedBf16 w{(const __nv_bfloat16*)w_out_bf16, s->C, 1};  // B(k=o, n=c) = Wout[o][c]
  return gemm(doA, w, StoreBf16Pair{dy, (__nv_bfloat16*)dy_bf16, nullptr, s->C}, T, s->C, K, 1,
              st);
}

int32_t ppf_sg_mse(const PpfSgShape* s, const float* out, const float* f_old, const float* f_new,
                   void* grad_bf16, double* loss, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw, K = 2LL * s->P * s->P;
  unsigned blocks;
  if ((rc = grid1d(T * K, &blocks))) return rc;
  mse_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, f_old, f_new,
                                                       (__nv_bfloat16*)grad_bf16, loss, T, s->P,
                                                       s->H, s->pitch, gh, gw, s->s0, s->s1,
                                                       1.0f / (float)(T * K));
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

int32_t ppf_sg_apply(const PpfSgShape* s, const float* out, const float* f_old, float* f_new,
                     void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  const int gh = s->H / s->P, gw = s->W / s->P;
  const long long T = (long long)s->B * gh * gw, K = 2LL * s->P * s->P;
  unsigned blocks;
  if ((rc = grid1d(T * K, &blocks))) return rc;
  apply_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, f_old, f_new, T, s->P, s->H,
                                                         s->pitch, gh, gw, 1.0f / s->s0,
                                                         1.0f / s->s1, s->lo0, s->hi0, s->lo1,
                                                         s->hi1);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// out[3 B] is overwritten.
int32_t ppf_sg_residual(const PpfSgShape* s, const float* u, const float* pred,
                        const float* stepped, int32_t k, double* out, void* stream) {
  clear_error();
  int32_t rc = sg_check(s);
  if (rc) return rc;
  if (!u || !pred || !stepped || !out || k < 1) return fail(PPF_ERR_INVALID, "bad residual args");
  const long long n = (long long)s->H * s->W;
  long long bx = (n + 255) / 256;
  if (bx > 1216) bx = 1216;  // 8 CTAs of 256 per SM over 152 SMs
  dim3 grid((unsigned)bx, (unsigned)s->B);
  PPF_TRY_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 3 * s->B, (cudaStream_t)stream));
  residual_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(u, pred, stepped, s->H, s->W, s->pitch,
                                                          (float)k, out);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// 1: GEMMs with K-contiguous operands run on tcgen05 (default); 0: mma.sync.
int32_t ppf_sg_set_tensor_path(int32_t tcgen05) {
  clear_error();
  g_tc_enabled = tcgen05 ? 1 : 0;
  return PPF_OK;
}

int32_t ppf_sg_cast_bf16(const float* x, void* y, long long n, void* stream) {
  clear_error();
  if (!x || !y) return fail(PPF_ERR_INVALID, "NULL pointer");
  unsigned blocks;
  int32_t rc = grid1d(n, &blocks);
  if (rc) return rc;
  cast_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(x, (__nv_bfloat16*)y, n);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

int32_t ppf_sg_adam(float* w, void* w_bf16, const float* g, float* m1, float* m2, long long n,
                    float lr, float b1, float b2, float eps, int32_t step, float weight_decay,
                    void* stream) {
  clear_error();
  if (!w || !g || !m1 || !m2 || step < 1) return fail(PPF_ERR_INVALID, "bad Adam arguments");
  unsigned blocks;
  int32_t rc = grid1d(n, &blocks);
  if (rc) return rc;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16*)w_bf16, g, m1, m2, n,
                                                        lr, b1, b2, eps, c1, c2, weight_decay);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

}  // extern "C"
