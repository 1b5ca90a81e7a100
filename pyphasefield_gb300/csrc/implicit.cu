// Implicit and Crank-Nicolson diffusion: pyphasefield's engines
// engine_ImplicitDiffusion{1,2,3}D[_ADI], engine_CrankNicolsonDiffusion{1,2,3}D[_ADI]
// and their *_GMRES twins (Engines/Diffusion.py:210-633), on periodic
// interior grids (the reference's matrices are periodic, Diffusion.py:18-196).
//
// Line solves (1-D engines and the ADI engines). Along one axis every line
// solves the periodic system (1 + 2a) x_i - a (x_{i-1} + x_{i+1}) = d_i. With
// r in (0, 1) the root of a r^2 - (1 + 2a) r + a = 0 the operator factors as
// (a / r)(I - r S)(I - r S^-1), S the cyclic shift, so
//   y_i = (r / a) d_i + r y_{i-1}   (cyclic forward recurrence)
//   x_i = y_i + r x_{i+1}           (cyclic backward recurrence)
// Both recurrences contract (|r| < 1). Each line is cut into segments; a
// segment's local sums with zero carry (pass 1), a short per-line pass that
// closes the cyclic carries in double (pass 2), and a pass that recomputes
// each segment from its true carries (pass 3) give the exact solution with
// three streaming kernels: 12 bytes of traffic per cell and float.
//   - lines along y or z: one thread per (column, 32-cell segment), threads
//     of a warp on adjacent columns, so every load and store is coalesced;
//   - lines along x: one warp per 256-cell segment, cell i of a 32-cell
//     chunk in lane i, the recurrence across lanes as a weighted warp scan.
// The Crank-Nicolson explicit half step (1 - 2a) c + a (c[-e] + c[+e]) along
// any axis e is folded into the right-hand side loads.
//
// Full systems (2-D and 3-D engines without ADI): the reference factors the
// dense N x N matrix. Here the Chebyshev semi-iteration runs on the 2d+1
// point operator, whose spectrum [1, 1 + 4 d a] is known in closed form, so
// the iteration count for a given error bound is fixed before the first
// iteration: one fused stencil kernel per iteration, no reductions.
#include <math.h>

#include "ppf_common.cuh"

namespace ppf {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSeg = 32;      // lines along y/z: cells per thread segment
constexpr int kLineThreads = 128;

template <typename T>
struct V2;
template <>
struct V2<float> {
  using type = float2;
};
template <>
struct V2<double> {
  using type = double2;
};

// Lines of one solve. Physical axes: x (contiguous), y (rows), z (planes).
struct Lines {
  int n;           // cells per line
  int nseg;        // segments per line
  int seglen;      // kSeg or kXSegV
  int nlines;
  int64_t stride;  // elements between consecutive cells of a line
  // lines along y or z: line = o * nx + x, o the remaining axis
  int nx, no;
  int64_t ostride;
  // lines along x: line = z * ny + y
  int ny;
  int64_t pitch, plane;
  // explicit part of the right-hand side
  int expl;        // 0 none, 1 along the solved axis, 2 along another axis
  int e_is_x;      // expl == 2 on y/z lines: the other axis is x (else the remaining one)
  int e_is_y;      // expl == 2 on x lines: the other axis is y (else z)
  int ne;          // extent of the explicit axis
  int64_t estride;
};

template <typename T>
struct LineCoef {
  T r, kappa;   // recurrence root and r / a (the recurrences run on d,
                // the solution is kappa times their result)
  T w0, w1;     // rhs = w0 c + w1 (c[-e] + c[+e])
  T rpow[33];   // r^0 .. r^32 (compile-time indices only)
  T rbit[8];    // r^1, r^2, r^4, ..., r^128
};

template <typename T>
struct CarryCoef {
  T R, G;       // r^L and sum_{k<L} r^(2k+1) of a full segment
  T Rl, Gl;     // the same for the last segment
  T inv_close;  // 1 / (1 - r^n)
  T Rp[6];      // R^1, R^2, R^4, R^8, R^16, R^32
};

// p[b] = q^(2^b), b < NB (compile-time indices only: a lane-dependent index
// into kernel parameters would serialise the warp on the constant cache).
// Returns q^e for 0 <= e < 2^NB.
template <int NB, typename T>
__device__ __forceinline__ T pow_bits(const T* p, int e) {
  T v = T(1);
#pragma unroll
  for (int b = 0; b < NB; ++b)
    if ((e >> b) & 1) v *= p[b];
  return v;
}

// Offsets of the two neighbours of coordinate q along an axis of extent n
// and stride st, periodic.
__device__ __forceinline__ void wrap_offsets(int q, int n, int64_t st, int64_t& om,
                                             int64_t& op) {
  om = (q == 0 ? (int64_t)(n - 1) : (int64_t)-1) * st;
  op = (q == n - 1 ? (int64_t)(1 - n) : (int64_t)1) * st;
}

// ---------------------------------------------------------------- y/z lines
// A thread takes one 32-cell segment of two adjacent columns (x, x + 1): one
// 8- or 16-byte load per cell pair, two independent recurrences.
struct StridedIdx {
  int x, o, s;
  int64_t base;
  bool ok, pair;
};

__device__ __forceinline__ StridedIdx strided_index(const Lines& L) {
  StridedIdx r;
  r.x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int64_t so = (int64_t)blockIdx.y + (int64_t)gridDim.y * blockIdx.z;
  r.ok = r.x < L.nx && so < (int64_t)L.nseg * L.no;
  r.pair = r.x + 1 < L.nx;
  r.s = (int)(so % L.nseg);
  r.o = (int)(so / L.nseg);
  r.base = r.x + (int64_t)r.o * L.ostride;
  return r;
}

// Two adjacent cells (the second 0 when the column does not exist); the
// offset is even, so the vector load is aligned.
template <typename T>
__device__ __forceinline__ void load2(const T* __restrict__ p, bool pair, T (&v)[2]) {
  if (pair) {
    if constexpr (sizeof(T) == 4) {
      const float2 q = __ldg(reinterpret_cast<const float2*>(p));
      v[0] = q.x, v[1] = q.y;
    } else {
      const double2 q = __ldg(reinterpret_cast<const double2*>(p));
      v[0] = q.x, v[1] = q.y;
    }
  } else {
    v[0] = __ldg(p);
    v[1] = T(0);
  }
}

template <typename T>
__device__ __forceinline__ void store2(T* p, bool pair, T a, T b) {
  if (pair) {
    if constexpr (sizeof(T) == 4)
      *reinterpret_cast<float2*>(p) = make_float2(a, b);
    else
      *reinterpret_cast<double2*>(p) = make_double2(a, b);
  } else {
    *p = a;
  }
}

// Offsets of the explicit part's neighbours, per column.
struct EOff {
  int64_t m[2], p[2];
};

template <int EXPL>
__device__ __forceinline__ EOff strided_eoffsets(const Lines& L, const StridedIdx& id) {
  EOff e{};
  if (EXPL == 2) {
    if (L.e_is_x) {
      wrap_offsets(id.x, L.ne, 1, e.m[0], e.p[0]);
      wrap_offsets(id.x + 1 < L.ne ? id.x + 1 : 0, L.ne, 1, e.m[1], e.p[1]);
    } else {
      wrap_offsets(id.o, L.ne, L.estride, e.m[0], e.p[0]);
      e.m[1] = e.m[0], e.p[1] = e.p[0];
    }
  }
  return e;
}

// Right-hand side of the cell pair at line position i (pointer p).
template <typename T, int EXPL>
__device__ __forceinline__ void rhs2(const T* __restrict__ p, const Lines& L,
                                     const LineCoef<T>& k, const StridedIdx& id, int i,
                                     const EOff& e, T (&d)[2]) {
  load2(p, id.pair, d);
  if (EXPL == 0) return;
  T a[2], b[2];
  if (EXPL == 1) {
    int64_t om, op;
    wrap_offsets(i, L.n, L.stride, om, op);
    load2(p + om, id.pair, a);
    load2(p + op, id.pair, b);
  } else if (L.e_is_x) {
    a[0] = __ldg(p + e.m[0]);
    b[0] = __ldg(p + e.p[0]);
    a[1] = id.pair ? __ldg(p + 1 + e.m[1]) : T(0);
    b[1] = id.pair ? __ldg(p + 1 + e.p[1]) : T(0);
  } else {
    load2(p + e.m[0], id.pair, a);
    load2(p + e.p[0], id.pair, b);
  }
#pragma unroll
  for (int c = 0; c < 2; ++c) d[c] = k.w0 * d[c] + k.w1 * (a[c] + b[c]);
}

// Pass 1: per segment, y's end value with zero carry (F) and the sum of
// r^(i - start) y_i over the segment (Bu).
template <typename T, int EXPL>
__global__ void __launch_bounds__(kLineThreads)
    line_sums_yz(Lines L, LineCoef<T> k, const T* __restrict__ in,
                 typename V2<T>::type* __restrict__ seg) {
  pdl_wait();
  pdl_launch_next();
  const StridedIdx id = strided_index(L);
  if (!id.ok) return;
  const EOff e = strided_eoffsets<EXPL>(L, id);
  const int i0 = id.s * kSeg;
  const int len = min(kSeg, L.n - i0);
  const T* p = in + id.base + (int64_t)i0 * L.stride;
  T d[kSeg][2];
  if (len == kSeg) {
#pragma unroll
    for (int j = 0; j < kSeg; ++j) rhs2<T, EXPL>(p + (int64_t)j * L.stride, L, k, id, i0 + j, e, d[j]);
  } else {
#pragma unroll
    for (int j = 0; j < kSeg; ++j) {
      if (j < len)
        rhs2<T, EXPL>(p + (int64_t)j * L.stride, L, k, id, i0 + j, e, d[j]);
      else
        d[j][0] = d[j][1] = T(0);
    }
  }
  T u0 = 0, u1 = 0, b0 = 0, b1 = 0;
#pragma unroll
  for (int j = 0; j < kSeg; ++j) {
    if (j < len) {
      u0 = fma(k.r, u0, d[j][0]);
      u1 = fma(k.r, u1, d[j][1]);
      b0 = fma(k.rpow[j], u0, b0);
      b1 = fma(k.rpow[j], u1, b1);
    }
  }
  typename V2<T>::type* q = seg + (int64_t)id.s * L.nlines + (int64_t)id.o * L.nx + id.x;
  q[0] = {u0, b0};
  if (id.pair) q[1] = {u1, b1};
}

// Pass 3: the segment again, from its true carries.
template <typename T, int EXPL>
__global__ void __launch_bounds__(kLineThreads)
    line_solve_yz(Lines L, LineCoef<T> k, const T* __restrict__ in,
                  const typename V2<T>::type* __restrict__ seg, T* __restrict__ out) {
  pdl_wait();
  pdl_launch_next();
  const StridedIdx id = strided_index(L);
  if (!id.ok) return;
  const EOff e = strided_eoffsets<EXPL>(L, id);
  const int i0 = id.s * kSeg;
  const int len = min(kSeg, L.n - i0);
  const int64_t off0 = id.base + (int64_t)i0 * L.stride;
  const typename V2<T>::type* q = seg + (int64_t)id.s * L.nlines + (int64_t)id.o * L.nx + id.x;
  const typename V2<T>::type c0 = q[0];
  const typename V2<T>::type c1 = id.pair ? q[1] : c0;
  T y[kSeg][2];
  if (len == kSeg) {
#pragma unroll
    for (int j = 0; j < kSeg; ++j)
      rhs2<T, EXPL>(in + off0 + (int64_t)j * L.stride, L, k, id, i0 + j, e, y[j]);
  } else {
#pragma unroll
    for (int j = 0; j < kSeg; ++j) {
      if (j < len)
        rhs2<T, EXPL>(in + off0 + (int64_t)j * L.stride, L, k, id, i0 + j, e, y[j]);
      else
        y[j][0] = y[j][1] = T(0);
    }
  }
  T y0 = c0.x, y1 = c1.x;
#pragma unroll
  for (int j = 0; j < kSeg; ++j) {
    y0 = fma(k.r, y0, y[j][0]);
    y1 = fma(k.r, y1, y[j][1]);
    y[j][0] = y0;
    y[j][1] = y1;
  }
  T x0 = c0.y, x1 = c1.y;
#pragma unroll
  for (int j = kSeg - 1; j >= 0; --j) {
    if (j < len) {
      x0 = fma(k.r, x0, y[j][0]);
      x1 = fma(k.r, x1, y[j][1]);
      store2(out + off0 + (int64_t)j * L.stride, id.pair, k.kappa * x0, k.kappa * x1);
    }
  }
}

// ---------------------------------------------------------------- x lines
// A warp takes a 512-cell segment of a row as 4 chunks of 128 cells, lane j
// holding cells 4j .. 4j+3 of a chunk (one 16-byte load). Within a lane the
// recurrence runs over its 4 cells; across lanes it is a warp scan with
// weights r^4, r^8, ... (5 shuffles per 4 cells).
constexpr int kXC = 4;            // chunks per segment
constexpr int kXSegV = 128 * kXC;  // cells per segment

struct XIdx {
  int line, s, lane;
  int64_t row;
  bool ok;
};

__device__ __forceinline__ XIdx x_index(const Lines& L) {
  XIdx r;
  r.lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (kLineThreads / 32) + (threadIdx.x >> 5);
  r.ok = w < (int64_t)L.nlines * L.nseg;  // uniform across the warp
  r.line = (int)(w / L.nseg);
  r.s = (int)(w % L.nseg);
  const int yy = r.line % L.ny, zz = r.line / L.ny;
  r.row = (int64_t)zz * L.plane + (int64_t)yy * L.pitch;
  return r;
}

// Cells i .. i+3 of a row (i a multiple of 4, so the 16 or 32 bytes are
// aligned: the pitch is a multiple of 4). Cells at or past n read 0; a
// vector that starts below n lies inside the row's pitch.
template <typename T>
__device__ __forceinline__ void load4(const T* __restrict__ row, int i, int n, T (&v)[4]) {
  if (i >= n) {
    v[0] = v[1] = v[2] = v[3] = T(0);
    return;
  }
  if constexpr (sizeof(T) == 4) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(row + i));
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
  } else {
    const double2 a = __ldg(reinterpret_cast<const double2*>(row + i));
    const double2 b = __ldg(reinterpret_cast<const double2*>(row + i + 2));
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
#pragma unroll
  for (int k = 1; k < 4; ++k)
    if (i + k >= n) v[k] = T(0);
}

// Right-hand side of the segment's cells: d[c][k] = cell 128c + 4 lane + k.
template <typename T, int EXPL>
__device__ __forceinline__ void x_rhs(const T* __restrict__ in, const Lines& L,
                                      const LineCoef<T>& k, const XIdx& id,
                                      T (&d)[kXC][4]) {
  const T* row = in + id.row;
  const int i0 = id.s * kXSegV;
#pragma unroll
  for (int c = 0; c < kXC; ++c) load4(row, i0 + 128 * c + 4 * id.lane, L.n, d[c]);
  if (EXPL == 0) return;
  if (EXPL == 2) {
    int64_t em, ep;
    const int yy = id.line % L.ny, zz = id.line / L.ny;
    wrap_offsets(L.e_is_y ? yy : zz, L.ne, L.estride, em, ep);
#pragma unroll
    for (int c = 0; c < kXC; ++c) {
      T a[4], b[4];
      const int i = i0 + 128 * c + 4 * id.lane;
      load4(row + em, i, L.n, a);
      load4(row + ep, i, L.n, b);
#pragma unroll
      for (int q = 0; q < 4; ++q) d[c][q] = k.w0 * d[c][q] + k.w1 * (a[q] + b[q]);
    }
    return;
  }
  // along the row itself: neighbours inside the lane, from the lanes and
  // chunks beside, or (segment and line ends) from memory; every lane takes
  // part in every shuffle
  const T lo_edge = __ldg(row + (i0 == 0 ? L.n - 1 : i0 - 1));
  const T hi_edge = __ldg(row + (i0 + kXSegV < L.n ? i0 + kXSegV : 0));
  const T first = __ldg(row);
  T left[kXC], right[kXC];
#pragma unroll
  for (int c = 0; c < kXC; ++c) {
    const T up = __shfl_up_sync(kFull, d[c][3], 1);
    const T dn = __shfl_down_sync(kFull, d[c][0], 1);
    const T prev_last = __shfl_sync(kFull, d[c > 0 ? c - 1 : 0][3], 31);
    const T next_first = __shfl_sync(kFull, d[c < kXC - 1 ? c + 1 : 0][0], 0);
    left[c] = id.lane > 0 ? up : (c > 0 ? prev_last : lo_edge);
    right[c] = id.lane < 31 ? dn : (c < kXC - 1 ? next_first : hi_edge);
  }
#pragma unroll
  for (int c = 0; c < kXC; ++c) {
    const int i = i0 + 128 * c + 4 * id.lane;
    T v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const T l = q > 0 ? d[c][q > 0 ? q - 1 : 0] : left[c];
      T rr = q < 3 ? d[c][q < 3 ? q + 1 : 0] : right[c];
      if (i + q == L.n - 1) rr = first;
      v[q] = i + q < L.n ? k.w0 * d[c][q] + k.w1 * (l + rr) : T(0);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) d[c][q] = v[q];
  }
}

// Inclusive scans over lanes with weight r^(4 * distance).
template <typename T>
__device__ __forceinline__ T scan4_up(T t, const LineCoef<T>& k, int lane) {
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    const T o = __shfl_up_sync(kFull, t, 1 << b);
    if (lane >= (1 << b)) t = fma(k.rbit[b + 2], o, t);
  }
  return t;
}

template <typename T>
__device__ __forceinline__ T scan4_down(T t, const LineCoef<T>& k, int lane) {
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    const T o = __shfl_down_sync(kFull, t, 1 << b);
    if (lane + (1 << b) < 32) t = fma(k.rbit[b + 2], o, t);
  }
  return t;
}

// Forward recurrence u_i = d_i + r u_{i-1} over one chunk entered with
// `carry` (the u before the chunk); returns the chunk's u in u[4] and the u
// of its last valid cell (nv valid cells, 1..128).
template <typename T>
__device__ __forceinline__ T x_forward(const T (&d)[4], T carry, int nv, T w4j,
                                       const LineCoef<T>& k, int lane, T (&u)[4]) {
  u[0] = d[0];
  u[1] = fma(k.r, u[0], d[1]);
  u[2] = fma(k.r, u[1], d[2]);
  u[3] = fma(k.r, u[2], d[3]);
  const T S = scan4_up(u[3], k, lane);
  const T prev = __shfl_up_sync(kFull, S, 1);
  const T yin = fma(w4j, carry, lane > 0 ? prev : T(0));  // u before the lane's cells
  T rp = k.r;
#pragma unroll
  for (int q = 0; q < 4; ++q, rp *= k.r) u[q] = fma(rp, yin, u[q]);
  if (nv == 128) return __shfl_sync(kFull, u[3], 31);
  const int q = (nv - 1) & 3;
  const T sel = q == 0 ? u[0] : q == 1 ? u[1] : q == 2 ? u[2] : u[3];
  return __shfl_sync(kFull, sel, (nv - 1) >> 2);
}

template <typename T, int EXPL>
__global__ void __launch_bounds__(kLineThreads)
    line_sums_x(Lines L, LineCoef<T> k, const T* __restrict__ in,
                typename V2<T>::type* __restrict__ seg) {
  pdl_wait();
  pdl_launch_next();
  const XIdx id = x_index(L);
  if (!id.ok) return;
  T d[kXC][4];
  x_rhs<T, EXPL>(in, L, k, id, d);
  const int i0 = id.s * kXSegV;
  const T w4j = pow_bits<5>(k.rbit + 2, id.lane);  // r^(4 lane)
  T carry = 0, bu = 0, pwk = 1;
#pragma unroll
  for (int c = 0; c < kXC; ++c) {
    const int nv = min(128, L.n - (i0 + 128 * c));
    if (nv > 0) {
      T u[4];
      const T last = x_forward(d[c], carry, nv, w4j, k, id.lane, u);
      const int base = 4 * id.lane;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (base + q >= nv) u[q] = T(0);
      T h = fma(k.r, u[3], u[2]);
      h = fma(k.r, h, u[1]);
      h = fma(k.r, h, u[0]);
      bu = fma(pwk * w4j, h, bu);
      carry = last;
      pwk *= k.rbit[7];
    }
  }
#pragma unroll
  for (int sh = 16; sh > 0; sh >>= 1) bu += __shfl_xor_sync(kFull, bu, sh);
  if (id.lane == 0) seg[(int64_t)id.s * L.nlines + id.line] = {carry, bu};
}

template <typename T, int EXPL>
__global__ void __launch_bounds__(kLineThreads)
    line_solve_x(Lines L, LineCoef<T> k, const T* __restrict__ in,
                 const typename V2<T>::type* __restrict__ seg, T* __restrict__ out) {
  pdl_wait();
  pdl_launch_next();
  const XIdx id = x_index(L);
  if (!id.ok) return;
  T y[kXC][4];
  x_rhs<T, EXPL>(in, L, k, id, y);
  const typename V2<T>::type cr = seg[(int64_t)id.s * L.nlines + id.line];
  const int i0 = id.s * kXSegV;
  const int base = 4 * id.lane;
  const T w4j = pow_bits<5>(k.rbit + 2, id.lane);        // r^(4 lane)
  const T w4t = pow_bits<5>(k.rbit + 2, 31 - id.lane);   // r^(4 (31 - lane))
  T carry = cr.x;
#pragma unroll
  for (int c = 0; c < kXC; ++c) {
    const int nv = min(128, L.n - (i0 + 128 * c));
    if (nv > 0) {
      T u[4];
      carry = x_forward(y[c], carry, nv, w4j, k, id.lane, u);
#pragma unroll
      for (int q = 0; q < 4; ++q) y[c][q] = base + q < nv ? u[q] : T(0);
    }
  }
  T* row = out + id.row;
  carry = cr.y;  // x just after the segment
#pragma unroll
  for (int c = kXC - 1; c >= 0; --c) {
    const int nv = min(128, L.n - (i0 + 128 * c));
    if (nv > 0) {
      T v[4];
      v[3] = y[c][3];
      v[2] = fma(k.r, v[3], y[c][2]);
      v[1] = fma(k.r, v[2], y[c][1]);
      v[0] = fma(k.r, v[1], y[c][0]);
      const T W = scan4_down(v[0], k, id.lane);
      const T nxt = __shfl_down_sync(kFull, W, 1);
      T after = id.lane < 31 ? nxt : T(0);  // x after the lane's cells, carry excluded
      if (nv == 128) after = fma(w4t, carry, after);
      T x[4];
      T rp = k.r;
#pragma unroll
      for (int q = 3; q >= 0; --q, rp *= k.r) x[q] = fma(rp, after, v[q]);
      if (nv < 128) {  // the carry enters after the last valid cell
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (base + q < nv) x[q] = fma(pow_bits<8>(k.rbit, nv - (base + q)), carry, x[q]);
      }
      carry = __shfl_sync(kFull, x[0], 0);
      const int i = i0 + 128 * c + base;
      if (base + 3 < nv) {
        if constexpr (sizeof(T) == 4) {
          *reinterpret_cast<float4*>(row + i) =
              make_float4(k.kappa * x[0], k.kappa * x[1], k.kappa * x[2], k.kappa * x[3]);
        } else {
          *reinterpret_cast<double2*>(row + i) = make_double2(k.kappa * x[0], k.kappa * x[1]);
          *reinterpret_cast<double2*>(row + i + 2) = make_double2(k.kappa * x[2], k.kappa * x[3]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (base + q < nv) row[i + q] = k.kappa * x[q];
      }
    }
  }
}

// ---------------------------------------------------------------- carries
// Pass 2, one warp per line: closes the two cyclic recurrences over the
// segments. In: (F_s, Bu_s). Out: (y just before segment s, x just after it).
// Over the segments the recurrences are Y_s = F_s + R Y_{s-1} and
// X_s = Bv_s + R X_{s+1} with Bv_s = Bu_s + G Y_{s-1} (the last segment has
// its own Rl, Gl); the warp runs them as weighted scans, 32 segments at a
// time, in the field's precision (both recurrences contract).
template <typename T>
__device__ __forceinline__ T wscan_up(T v, const T* Rp, int lane) {
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    const T o = __shfl_up_sync(kFull, v, 1 << b);
    if (lane >= (1 << b)) v = fma(Rp[b], o, v);
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T wscan_down(T v, const T* Rp, int lane) {
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    const T o = __shfl_down_sync(kFull, v, 1 << b);
    if (lane + (1 << b) < 32) v = fma(Rp[b], o, v);
  }
  return v;
}

template <typename T>
__global__ void __launch_bounds__(128)
    line_carry(Lines L, CarryCoef<T> cc, typename V2<T>::type* __restrict__ seg) {
  pdl_wait();
  pdl_launch_next();
  const int lane = threadIdx.x & 31;
  const int line = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (line >= L.nlines) return;  // uniform across the warp
  const int m = L.nseg, mc = m - 1;  // segments 0 .. mc-1 share R and G
  auto at = [&](int s) -> typename V2<T>::type& { return seg[(int64_t)s * L.nlines + line]; };
  const T up_w = pow_bits<6>(cc.Rp, lane + 1);   // R^(lane+1)
  const T dn_w = pow_bits<6>(cc.Rp, 32 - lane);  // R^(32-lane)
  // forward chain from `start` (the y before segment 0); calls f(s, y_before)
  auto forward = [&](T start, auto&& f) -> T {
    T carry = start;
    for (int b0 = 0; b0 < mc; b0 += 32) {
      const int s = b0 + lane;
      const int nv = min(32, mc - b0);
      const T v = s < mc ? at(s).x : 0.0;
      const T y = fma(up_w, carry, wscan_up(v, cc.Rp, lane));
      const T prev = __shfl_up_sync(kFull, y, 1);  // every lane takes part
      const T before = lane == 0 ? carry : prev;
      if (s < mc) f(s, before);
      carry = __shfl_sync(kFull, y, nv - 1);
    }
    return carry;  // y before the last segment
  };
  // the y of the line's last cell with zero start, then the true start
  const T y_mc0 = forward(0.0, [](int, T) {});
  const T ystart = (at(mc).x + cc.Rl * y_mc0) * cc.inv_close;
  const T y_mc = forward(ystart, [&](int s, T before) {
    typename V2<T>::type& v = at(s);
    v.y = (v.y + before * cc.G);  // Bu -> Bv
    v.x = before;                          // F -> y before the segment
  });
  __syncwarp();
  {
    typename V2<T>::type& v = at(mc);
    if (lane == 0) {
      v.y = (v.y + y_mc * cc.Gl);
      v.x = y_mc;
    }
  }
  __syncwarp();
  // backward chain over segments mc-1 .. 0 from `start` (the x after
  // segment mc-1, i.e. the first x of the last segment); calls g(s, x_after)
  auto backward = [&](T start, auto&& g) -> T {
    T carry = start;
    for (int top = mc; top > 0; top -= 32) {
      const int s = top - 32 + lane;  // batches end at top; padding at the low end
      const int first = max(0, top - 32) - (top - 32);  // first valid lane
      const T v = s >= 0 ? at(s).y : 0.0;
      const T x = fma(dn_w, carry, wscan_down(v, cc.Rp, lane));
      const T next = __shfl_down_sync(kFull, x, 1);  // every lane takes part
      const T after = lane == 31 ? carry : next;
      if (s >= 0) g(s, after);
      carry = __shfl_sync(kFull, x, first);
    }
    return carry;  // x of the line's first cell
  };
  const T bv_last = at(mc).y;
  // zero start after the line's end: x_0 = (sum ...) / (1 - r^n)
  const T x_first0 = backward(bv_last, [](int, T) {});
  const T x0 = x_first0 * cc.inv_close;
  const T x_last = bv_last + cc.Rl * x0;  // first x of the last segment
  __syncwarp();
  backward(x_last, [&](int s, T after) { at(s).y = after; });
  if (lane == 0) at(mc).y = x0;
}

// The same pass with the line's (F, Bu) held in registers: B batches of 32
// segments per lane, one load and one store round (lines of up to 32 B + 1
// segments). Batches are aligned at segment 0; the top batch may be partial
// (nv valid lanes), so the backward chain enters it at lane nv - 1.
template <typename T, int B>
__global__ void __launch_bounds__(128)
    line_carry_reg(Lines L, CarryCoef<T> cc, typename V2<T>::type* __restrict__ seg) {
  pdl_wait();
  pdl_launch_next();
  const int lane = threadIdx.x & 31;
  const int line = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (line >= L.nlines) return;  // uniform across the warp
  const int mc = L.nseg - 1;     // segments 0 .. mc-1 share R and G
  const int nb = (mc + 31) / 32;
  typename V2<T>::type* col = seg + line;
  const int64_t st = L.nlines;
  T F[B], Bv[B], Yin[B], Xin[B];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int s = 32 * b + lane;
    F[b] = Bv[b] = T(0);
    if (b < nb && s < mc) {
      const typename V2<T>::type v = col[s * st];
      F[b] = v.x;
      Bv[b] = v.y;
    }
  }
  const typename V2<T>::type last = col[(int64_t)mc * st];
  const T up_w = pow_bits<6>(cc.Rp, lane + 1);   // R^(lane+1)
  const T dn_w = pow_bits<6>(cc.Rp, 32 - lane);  // R^(32-lane)
  T carry = T(0);
#pragma unroll
  for (int b = 0; b < B; ++b) {
    if (b < nb) {
      const int nv = min(32, mc - 32 * b);
      const T y = fma(up_w, carry, wscan_up(F[b], cc.Rp, lane));
      carry = __shfl_sync(kFull, y, nv - 1);
    }
  }
  const T ystart = (last.x + cc.Rl * carry) * cc.inv_close;  // y of the line's last cell
  carry = ystart;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    if (b < nb) {
      const int nv = min(32, mc - 32 * b);
      const T y = fma(up_w, carry, wscan_up(F[b], cc.Rp, lane));
      const T prev = __shfl_up_sync(kFull, y, 1);
      Yin[b] = lane == 0 ? carry : prev;
      if (32 * b + lane < mc) Bv[b] = fma(Yin[b], cc.G, Bv[b]);
      carry = __shfl_sync(kFull, y, nv - 1);
    }
  }
  const T y_mc = carry;                          // y before the last segment
  const T bv_last = last.y + y_mc * cc.Gl;
  auto backward = [&](T start, bool keep) -> T {
    T c = start;
#pragma unroll
    for (int b = B - 1; b >= 0; --b) {
      if (b < nb) {
        const int nv = min(32, mc - 32 * b);
        const T w = nv == 32 ? dn_w : (lane < nv ? pow_bits<6>(cc.Rp, nv - lane) : T(0));
        const T x = fma(w, c, wscan_down(Bv[b], cc.Rp, lane));
        const T nxt = __shfl_down_sync(kFull, x, 1);
        if (keep) Xin[b] = lane == nv - 1 ? c : nxt;
        c = __shfl_sync(kFull, x, 0);
      }
    }
    return c;
  };
  const T x0 = backward(bv_last, false) * cc.inv_close;  // x of the line's first cell
  backward(bv_last + cc.Rl * x0, true);
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int s = 32 * b + lane;
    if (b < nb && s < mc) col[s * st] = {Yin[b], Xin[b]};
  }
  if (lane == 0) col[(int64_t)mc * st] = {y_mc, x0};
}

// ---------------------------------------------------------------- Chebyshev
// One iteration: y_new = y_prev + omega (y + gamma (b - A y) - y_prev), or
// y + gamma (b - A y) for the first. A y = diag y - a sum(neighbours of y);
// b = c, or for Crank-Nicolson w0 c + w1 sum(neighbours of c). y_new may
// alias y_prev (each cell reads its own y_prev only).
template <typename T>
struct ChebStep {
  T diag, a, w0, w1, gamma, omega;
  int first;
};

template <typename T, int ND, bool CN>
__global__ void __launch_bounds__(256)
    chebyshev_kernel(Geo g, ChebStep<T> k, const T* __restrict__ c, const T* __restrict__ y,
                     const T* yprev, T* ynew) {
  pdl_wait();
  pdl_launch_next();
  const int nx = g.n[ND - 1], ny = g.n[ND - 2];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  const int z = ND == 3 ? blockIdx.z : 0;
  const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
  int64_t zm = 0, zp = 0;
  if (ND == 3) {
    const int nz = g.n[0];
    zm = (int64_t)(z == 0 ? nz - 1 : z - 1) * g.plane;
    zp = (int64_t)(z == nz - 1 ? 0 : z + 1) * g.plane;
  }
  const int64_t zb = (int64_t)z * g.plane;
  for (int yy = blockIdx.y; yy < ny; yy += gridDim.y) {
    const int64_t ym = (int64_t)(yy == 0 ? ny - 1 : yy - 1) * g.pitch;
    const int64_t yp = (int64_t)(yy == ny - 1 ? 0 : yy + 1) * g.pitch;
    const int64_t yb = (int64_t)yy * g.pitch;
    const int64_t i = zb + yb + x;
    T sy = __ldg(y + zb + yb + xm) + __ldg(y + zb + yb + xp) + __ldg(y + zb + ym + x) +
           __ldg(y + zb + yp + x);
    if (ND == 3) sy += __ldg(y + zm + yb + x) + __ldg(y + zp + yb + x);
    const T yc = __ldg(y + i);
    T b = __ldg(c + i);
    if (CN) {
      T sc = __ldg(c + zb + yb + xm) + __ldg(c + zb + yb + xp) + __ldg(c + zb + ym + x) +
             __ldg(c + zb + yp + x);
      if (ND == 3) sc += __ldg(c + zm + yb + x) + __ldg(c + zp + yb + x);
      b = k.w0 * b + k.w1 * sc;
    }
    const T rich = yc + k.gamma * (b - (k.diag * yc - k.a * sy));
    ynew[i] = k.first ? rich : yprev[i] + k.omega * (rich - yprev[i]);
  }
}

// ---------------------------------------------------------------- host side
int phys_axis(const Geo& g, int axis) { return axis + (3 - g.ndim); }  // 0 z, 1 y, 2 x

struct Extents {
  int n[3];        // z, y, x
  int64_t st[3];   // strides
};

Extents extents(const Geo& g) {
  Extents e;
  e.n[0] = g.ndim == 3 ? g.n[0] : 1;
  e.n[1] = g.n[g.ndim - 2];
  e.n[2] = g.n[g.ndim - 1];
  e.st[0] = g.ndim == 3 ? g.plane : (int64_t)g.pitch * e.n[1];
  e.st[1] = g.pitch;
  e.st[2] = 1;
  return e;
}

Lines make_lines(const Geo& g, int axis) {
  const Extents e = extents(g);
  const int p = phys_axis(g, axis);
  Lines L{};
  L.n = e.n[p];
  L.stride = e.st[p];
  L.pitch = g.pitch;
  L.plane = e.st[0];
  L.ny = e.n[1];
  L.nx = e.n[2];
  if (p == 2) {
    L.seglen = kXSegV;
    L.nlines = e.n[0] * e.n[1];
  } else {
    L.seglen = kSeg;
    const int o = p == 1 ? 0 : 1;  // the remaining axis
    L.no = e.n[o];
    L.ostride = e.st[o];
    L.nlines = e.n[2] * L.no;
  }
  L.nseg = (L.n + L.seglen - 1) / L.seglen;
  return L;
}

size_t line_scratch_bytes(const Geo& g, int axis, int elem_bytes) {
  const Lines L = make_lines(g, axis);
  return (size_t)L.nlines * L.nseg * 2 * elem_bytes;
}

double recurrence_root(double a) { return 2.0 * a / (1.0 + 2.0 * a + sqrt(1.0 + 4.0 * a)); }

template <typename T>
int32_t copy_field(const Geo& g, const T* in, T* out, cudaStream_t st) {
  const Extents e = extents(g);
  const size_t bytes = (size_t)e.st[0] * e.n[0] * sizeof(T);
  PPF_TRY_CUDA(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, st));
  return PPF_OK;
}

template <typename T>
cudaError_t launch_carry(const Lines& L, const CarryCoef<T>& cc, typename V2<T>::type* seg,
                         cudaStream_t st) {
  const dim3 grid((L.nlines + 3) / 4), block(128);
  const int nb = (L.nseg - 1 + 31) / 32;
  if (nb <= 1) return launch(line_carry_reg<T, 1>, grid, block, 0, st, true, L, cc, seg);
  if (nb <= 2) return launch(line_carry_reg<T, 2>, grid, block, 0, st, true, L, cc, seg);
  if (nb <= 4) return launch(line_carry_reg<T, 4>, grid, block, 0, st, true, L, cc, seg);
  if (nb <= 8) return launch(line_carry_reg<T, 8>, grid, block, 0, st, true, L, cc, seg);
  if (nb <= 16) return launch(line_carry_reg<T, 16>, grid, block, 0, st, true, L, cc, seg);
  return launch(line_carry<T>, grid, block, 0, st, true, L, cc, seg);
}

template <typename T, int EXPL>
int32_t launch_line(const Lines& L, const LineCoef<T>& k, const CarryCoef<T>& cc, const T* in,
                    T* out, typename V2<T>::type* seg, cudaStream_t st) {
  if (L.seglen == kXSegV) {
    const int64_t warps = (int64_t)L.nlines * L.nseg;
    const dim3 grid((unsigned)((warps + kLineThreads / 32 - 1) / (kLineThreads / 32)));
    if (grid.x > 0x7fffffffu) return fail(PPF_ERR_INVALID, "grid too large");
    PPF_TRY_CUDA(launch(line_sums_x<T, EXPL>, grid, dim3(kLineThreads), 0, st, true, L, k, in, seg));
    PPF_TRY_CUDA(launch_carry<T>(L, cc, seg, st));
    PPF_TRY_CUDA(
        launch(line_solve_x<T, EXPL>, grid, dim3(kLineThreads), 0, st, true, L, k, in, seg, out));
    return PPF_OK;
  }
  const int64_t so = (int64_t)L.nseg * L.no;
  const unsigned gy = (unsigned)(so < 65535 ? so : 65535);
  const unsigned gz = (unsigned)((so + gy - 1) / gy);
  if (gz > 65535) return fail(PPF_ERR_INVALID, "grid too large for the line solver");
  const int pairs = (L.nx + 1) / 2;
  const dim3 grid((pairs + kLineThreads - 1) / kLineThreads, gy, gz);
  PPF_TRY_CUDA(launch(line_sums_yz<T, EXPL>, grid, dim3(kLineThreads), 0, st, true, L, k, in, seg));
  PPF_TRY_CUDA(launch_carry<T>(L, cc, seg, st));
  PPF_TRY_CUDA(
      launch(line_solve_yz<T, EXPL>, grid, dim3(kLineThreads), 0, st, true, L, k, in, seg, out));
  return PPF_OK;
}

// One periodic line solve along `axis` (C order) with an optional explicit
// half step along `eaxis` (-1: none) folded into the right-hand side.
template <typename T>
int32_t line_sweep(const Geo& g, int axis, double a, int eaxis, double ea, const T* in, T* out,
                   void* scratch, size_t scratch_bytes, cudaStream_t st) {
  if (axis < 0 || axis >= g.ndim) return fail(PPF_ERR_INVALID, "axis %d out of range", axis);
  if (eaxis >= g.ndim) return fail(PPF_ERR_INVALID, "explicit axis %d out of range", eaxis);
  if (!(a >= 0) || !isfinite(a) || !(ea >= 0) || !isfinite(ea))
    return fail(PPF_ERR_INVALID, "alpha must be finite and >= 0");
  Lines L = make_lines(g, axis);
  if (L.n < 3)
    return fail(PPF_ERR_INVALID,
                "periodic line solves need >= 3 cells along the solved axis (got %d)", L.n);
  if (eaxis >= 0 && in == out)
    return fail(PPF_ERR_INVALID, "in and out must differ when an explicit part is folded in");
  const size_t need = line_scratch_bytes(g, axis, sizeof(T));
  if (!scratch || scratch_bytes < need)
    return fail(PPF_ERR_INVALID, "scratch of %zu bytes needed (got %zu)", need, scratch_bytes);
  const Extents e = extents(g);
  LineCoef<T> k{};
  int mode = 0;
  k.w0 = T(1);
  k.w1 = T(0);
  if (eaxis >= 0) {
    const int pe = phys_axis(g, eaxis), pa = phys_axis(g, axis);
    if (e.n[pe] < 3 && pe != pa)
      return fail(PPF_ERR_INVALID, "the explicit axis needs >= 3 cells (got %d)", e.n[pe]);
    k.w0 = (T)(1.0 - 2.0 * ea);
    k.w1 = (T)ea;
    mode = pe == pa ? 1 : 2;
    L.ne = e.n[pe];
    L.estride = e.st[pe];
    L.e_is_x = pe == 2;
    L.e_is_y = pe == 1;
  }
  L.expl = mode;
  if (a == 0.0) {
    if (mode == 0) return in == out ? PPF_OK : copy_field(g, in, out, st);
    // the explicit half step alone: a line solve with a vanishing implicit part
  }
  const double r = a > 0 ? recurrence_root(a) : 0.0;
  k.r = (T)r;
  k.kappa = (T)(a > 0 ? r / a : 1.0);
  double pw = 1.0;
  for (int i = 0; i <= 32; ++i, pw *= r) k.rpow[i] = (T)pw;
  CarryCoef<T> cc{};
  const int Ll = L.n - (L.nseg - 1) * L.seglen;
  const double R = pow(r, L.seglen);
  cc.R = (T)R;
  cc.Rl = (T)pow(r, Ll);
  cc.G = (T)(r * (1.0 - pow(r, 2.0 * L.seglen)) / (1.0 - r * r));
  cc.Gl = (T)(r * (1.0 - pow(r, 2.0 * Ll)) / (1.0 - r * r));
  cc.inv_close = (T)(1.0 / (1.0 - pow(r, L.n)));
  for (int b = 0; b < 6; ++b) cc.Rp[b] = (T)pow(R, (double)(1 << b));
  for (int b = 0; b < 8; ++b) k.rbit[b] = (T)pow(r, (double)(1 << b));
  auto* seg = static_cast<typename V2<T>::type*>(scratch);
  switch (mode) {
    case 0: return launch_line<T, 0>(L, k, cc, in, out, seg, st);
    case 1: return launch_line<T, 1>(L, k, cc, in, out, seg, st);
    default: return launch_line<T, 2>(L, k, cc, in, out, seg, st);
  }
}

struct ChebPlan {
  int iters;
  double gamma, rho;
};

ChebPlan chebyshev_plan(double a, int ndim, double tol) {
  ChebPlan p{};
  const double lmax = 1.0 + 4.0 * ndim * a;
  p.gamma = 2.0 / (lmax + 1.0);
  p.rho = (lmax - 1.0) / (lmax + 1.0);
  if (p.rho <= 0) return p;
  const double need = 2.0 * fmax(1.0, 8.0 * ndim * a) / tol;
  p.iters = (int)ceil(acosh(need) / acosh(1.0 / p.rho));
  if (p.iters < 1) p.iters = 1;
  return p;
}

// Solve (1 + 2 d a) x - a sum(neighbours of x) = b on the periodic grid,
// b = in (rhs_a = 0) or (1 - 2 d rhs_a) in + rhs_a sum(neighbours of in).
template <typename T>
int32_t periodic_solve(const Geo& g, double a, double rhs_a, double tol, const T* in, T* out,
                       T* tmp, int32_t* iterations, cudaStream_t st) {
  if (!(a >= 0) || !isfinite(a) || !(rhs_a >= 0) || !isfinite(rhs_a))
    return fail(PPF_ERR_INVALID, "alpha must be finite and >= 0");
  if (!(tol > 0) || !(tol < 1)) return fail(PPF_ERR_INVALID, "tol must be in (0, 1)");
  for (int ax = 0; ax < g.ndim; ++ax)
    if (g.n[ax] < 3)
      return fail(PPF_ERR_INVALID, "periodic solves need >= 3 cells per axis (axis %d has %d)",
                  ax, g.n[ax]);
  if (!tmp || tmp == in || tmp == out || in == out)
    return fail(PPF_ERR_INVALID, "in, out and tmp must be three distinct buffers");
  const ChebPlan plan = chebyshev_plan(a, g.ndim, tol);
  const int d = g.ndim;
  ChebStep<T> k{};
  k.diag = (T)(1.0 + 2.0 * d * a);
  k.a = (T)a;
  k.w0 = (T)(1.0 - 2.0 * d * rhs_a);
  k.w1 = (T)rhs_a;
  k.gamma = (T)plan.gamma;
  const bool cn = rhs_a != 0.0;
  const Extents e = extents(g);
  const dim3 grid((e.n[2] + 255) / 256, (unsigned)(e.n[1] < 65535 ? e.n[1] : 65535),
                  (unsigned)e.n[0]);
  if (e.n[0] > 65535) return fail(PPF_ERR_INVALID, "too many planes");
  if (iterations) *iterations = plan.iters;
  auto run = [&](const ChebStep<T>& kk, const T* y, const T* yp, T* yn) -> int32_t {
    cudaError_t err;
    if (d == 2)
      err = cn ? launch(chebyshev_kernel<T, 2, true>, grid, dim3(256), 0, st, true, g, kk, in, y,
                        yp, yn)
               : launch(chebyshev_kernel<T, 2, false>, grid, dim3(256), 0, st, true, g, kk, in,
                        y, yp, yn);
    else
      err = cn ? launch(chebyshev_kernel<T, 3, true>, grid, dim3(256), 0, st, true, g, kk, in, y,
                        yp, yn)
               : launch(chebyshev_kernel<T, 3, false>, grid, dim3(256), 0, st, true, g, kk, in,
                        y, yp, yn);
    PPF_TRY_CUDA(err);
    return PPF_OK;
  };
  if (plan.iters == 0) {  // a = 0: x = b, as one step y + (b - y) from y = in
    ChebStep<T> k0 = k;
    k0.diag = T(1);
    k0.a = T(0);
    k0.gamma = T(1);
    k0.first = 1;
    return run(k0, in, nullptr, out);
  }
  // iterations j = 1..K; y_j lands in out when K - j is even, else in tmp
  const T* prev = nullptr;
  const T* cur = in;
  double om = 1.0;
  const double rho2 = plan.rho * plan.rho;
  for (int j = 1; j <= plan.iters; ++j) {
    if (j == 2)
      om = 2.0 / (2.0 - rho2);
    else if (j > 2)
      om = 1.0 / (1.0 - rho2 * om / 4.0);
    T* dst = ((plan.iters - j) % 2 == 0) ? out : tmp;
    ChebStep<T> kj = k;
    kj.first = j == 1;
    kj.omega = (T)om;
    const int32_t rc = run(kj, cur, prev, dst);
    if (rc) return rc;
    prev = cur;
    cur = dst;
  }
  return PPF_OK;
}

template <typename T>
int32_t implicit_step(const PpfImplicitDiffusionParams* p, const PpfGrid* grid, const T* in,
                      T* out, T* tmp, void* scratch, size_t scratch_bytes, int32_t* iterations,
                      void* stream) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (in == out) return fail(PPF_ERR_INVALID, "in and out must differ");
  if (!(p->dx > 0) || !(p->dt >= 0) || !(p->D >= 0) || !isfinite(p->dx) || !isfinite(p->dt) ||
      !isfinite(p->D))
    return fail(PPF_ERR_INVALID, "dx > 0, dt >= 0 and D >= 0 are required");
  const bool cn = p->solver == PPF_SOLVER_CRANK_NICOLSON;
  if (!cn && p->solver != PPF_SOLVER_IMPLICIT)
    return fail(PPF_ERR_INVALID, "solver must be PPF_SOLVER_IMPLICIT or PPF_SOLVER_CRANK_NICOLSON");
  const double a = (cn ? 0.5 : 1.0) * p->D * p->dt / (p->dx * p->dx);
  cudaStream_t st = (cudaStream_t)stream;
  if (iterations) *iterations = 0;
  const bool oned = g.ndim == 2 && g.n[0] == 1;
  if (oned) {  // engine_*Diffusion1D: one line along x
    return line_sweep<T>(g, 1, a, cn ? 1 : -1, a, in, out, scratch, scratch_bytes, st);
  }
  if (!p->adi) {
    const double tol = p->tol > 0 ? p->tol : (sizeof(T) == 4 ? 1e-7 : 1e-14);
    return periodic_solve<T>(g, a, cn ? a : 0.0, tol, in, out, tmp, iterations, st);
  }
  // ADI: the reference's axis order (Diffusion.py:428-431, 474-482, 527-533, 580-591)
  int sweeps[3][2];
  int ns = 0;
  if (!cn) {
    for (int ax = g.ndim - 1; ax >= 0; --ax) sweeps[ns][0] = ax, sweeps[ns][1] = -1, ++ns;
  } else if (g.ndim == 2) {
    sweeps[0][0] = 0, sweeps[0][1] = 0;
    sweeps[1][0] = 1, sweeps[1][1] = 1;
    ns = 2;
  } else {
    sweeps[0][0] = 1, sweeps[0][1] = 0;
    sweeps[1][0] = 0, sweeps[1][1] = 1;
    sweeps[2][0] = 2, sweeps[2][1] = 2;
    ns = 3;
  }
  if (cn && (!tmp || tmp == in || tmp == out))
    return fail(PPF_ERR_INVALID, "Crank-Nicolson ADI needs a tmp field distinct from in and out");
  const T* src = in;
  for (int i = 0; i < ns; ++i) {
    // without an explicit part a sweep may run in place: every thread reads
    // only the cells it writes after pass 1 has read them all
    T* dst = cn ? (((ns - 1 - i) % 2 == 0) ? out : tmp) : out;
    rc = line_sweep<T>(g, sweeps[i][0], a, sweeps[i][1], a, src, dst, scratch, scratch_bytes, st);
    if (rc) return rc;
    src = dst;
  }
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_implicit_scratch_bytes(const PpfGrid* grid, int32_t elem_bytes, size_t* bytes) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!bytes) return fail(PPF_ERR_INVALID, "bytes is NULL");
  if (elem_bytes != 4 && elem_bytes != 8) return fail(PPF_ERR_INVALID, "elem_bytes must be 4 or 8");
  size_t m = 0;
  for (int ax = 0; ax < g.ndim; ++ax) {
    const size_t b = line_scratch_bytes(g, ax, elem_bytes);
    m = b > m ? b : m;
  }
  *bytes = m;
  return PPF_OK;
}

int32_t ppf_line_solve_f32(const PpfGrid* grid, int32_t axis, double alpha, int32_t expl_axis,
                           double expl_alpha, const float* in, float* out, void* scratch,
                           size_t scratch_bytes, void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  return line_sweep<float>(g, axis, alpha, expl_axis, expl_alpha, in, out, scratch, scratch_bytes,
                           (cudaStream_t)stream);
}

int32_t ppf_line_solve_f64(const PpfGrid* grid, int32_t axis, double alpha, int32_t expl_axis,
                           double expl_alpha, const double* in, double* out, void* scratch,
                           size_t scratch_bytes, void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  return line_sweep<double>(g, axis, alpha, expl_axis, expl_alpha, in, out, scratch,
                            scratch_bytes, (cudaStream_t)stream);
}

int32_t ppf_periodic_solve_f32(const PpfGrid* grid, double alpha, double rhs_alpha, double tol,
                               const float* in, float* out, float* tmp, int32_t* iterations,
                               void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  return periodic_solve<float>(g, alpha, rhs_alpha, tol, in, out, tmp, iterations,
                               (cudaStream_t)stream);
}

int32_t ppf_periodic_solve_f64(const PpfGrid* grid, double alpha, double rhs_alpha, double tol,
                               const double* in, double* out, double* tmp, int32_t* iterations,
                               void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  return periodic_solve<double>(g, alpha, rhs_alpha, tol, in, out, tmp, iterations,
                                (cudaStream_t)stream);
}

int32_t ppf_diffusion_implicit_step_f32(const PpfImplicitDiffusionParams* p, const PpfGrid* g,
                                        const float* in, float* out, float* tmp, void* scratch,
                                        size_t scratch_bytes, int32_t* iterations, void* stream) {
  return implicit_step<float>(p, g, in, out, tmp, scratch, scratch_bytes, iterations, stream);
}

int32_t ppf_diffusion_implicit_step_f64(const PpfImplicitDiffusionParams* p, const PpfGrid* g,
                                        const double* in, double* out, double* tmp, void* scratch,
                                        size_t scratch_bytes, int32_t* iterations, void* stream) {
  return implicit_step<double>(p, g, in, out, tmp, scratch, scratch_bytes, iterations, stream);
}

}  // extern "C"
