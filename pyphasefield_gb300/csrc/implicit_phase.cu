// Implicit, Crank-Nicolson and IMEX Allen-Cahn ("CahnAllen") and
// Cahn-Hilliard engines (Engines/CahnAllen.py:137-267,
// Engines/CahnHilliard.py:148-341), dispatched as CahnAllen.simulation_loop
// (:325-361) and CahnHilliard.simulation_loop (:382-421) do.
//
// Their systems are periodic tridiagonal along a line with a diagonal that
// varies per cell (d_i = 1 + 2a + c (4 phi_i^2 - 6 phi_i + 2), the
// linearised double well) and constant off-diagonals -a. Line solves use
// the partition method with separators: the last cell of every 32-cell
// segment is a separator; the interior cells of a segment depend only on the
// separators on either side, so
//   pass 1 (a thread per segment) solves the interior block three times in
//          registers (right-hand side; unit coupling to the left separator;
//          to the right one) by forward and backward elimination and keeps
//          the end values,
//   pass 2 (a thread per line) solves the cyclic tridiagonal system of the
//          separators (Thomas with the Sherman-Morrison correction),
//   pass 3 (a thread per segment) solves the interior block once more with
//          its true separator values and writes the line.
// The full 2-D system of the GMRES engine runs the Chebyshev semi-iteration
// with Jacobi scaling (spectrum bound from the smallest possible diagonal),
// and the 1-D Cahn-Hilliard engines (a cyclic pentadiagonal system with
// row-dependent coefficients, one line) a banded elimination with the
// Woodbury correction for the periodic corners.
#include <math.h>

#include "ppf_common.cuh"
#include "ppf_grid.cuh"

namespace ppf {
namespace {

constexpr int kPSeg = 32;       // cells per segment; the last one is the separator
constexpr int kPThreads = 128;
constexpr int kRec = 8;         // values per segment record

// Geometry of the lines along one axis (physical axes z, y, x).
struct PLines {
  int n;            // cells per line
  int nseg;         // segments per line
  int nlines;
  int64_t stride;   // elements between the cells of a line
  int xfast;        // 1: lines along y/z, threads of a warp on adjacent columns
  int nx, no;       // y/z lines: line = o * nx + x
  int64_t ostride;
  int ny;           // x lines: line = z * ny + y
  int64_t pitch, plane;
};

template <typename T>
struct PCoef {
  T a;          // off-diagonal magnitude
  T dbase, dc;  // d_i = dbase + dc (4 b^2 - 6 b + 2), b the right-hand side
  T w0, w1;     // right-hand side b = w0 c + w1 (c[-1] + c[+1]) along the line (expl)
  int expl;     // 0: b = c
  const T* dvec;  // non-null: d_i = dvec[i] (one diagonal shared by every line)
};

__device__ __forceinline__ int64_t line_base(const PLines& L, int line) {
  if (L.xfast) {
    const int x = line % L.nx, o = line / L.nx;
    return x + (int64_t)o * L.ostride;
  }
  const int y = line % L.ny, z = line / L.ny;
  return (int64_t)z * L.plane + (int64_t)y * L.pitch;
}

// (line, segment) of this thread; y/z lines put adjacent columns in a warp,
// x lines adjacent segments of a row.
__device__ __forceinline__ bool seg_index(const PLines& L, int& line, int& s) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)L.nlines * L.nseg) return false;
  if (L.xfast) {
    const int64_t per = (int64_t)L.nx;  // lines of one `o` are nx consecutive threads
    const int64_t o = t / (per * L.nseg);
    const int64_t r = t - o * per * L.nseg;
    s = (int)(r / per);
    line = (int)(o * per + r % per);
  } else {
    line = (int)(t / L.nseg);
    s = (int)(t % L.nseg);
  }
  return true;
}

template <typename T>
__device__ __forceinline__ T rhs_val(const T* __restrict__ row, const PLines& L,
                                     const PCoef<T>& k, int i) {
  const T c = __ldg(row + (int64_t)i * L.stride);
  if (!k.expl) return c;
  const int im = i == 0 ? L.n - 1 : i - 1, ip = i == L.n - 1 ? 0 : i + 1;
  return k.w0 * c + k.w1 * (__ldg(row + (int64_t)im * L.stride) + __ldg(row + (int64_t)ip * L.stride));
}

// Correctly rounded reciprocal (the pivots of the eliminations).
__device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp(double x) { return __drcp_rn(x); }

// The segment's cells as 16-byte vectors (rows are 16-byte aligned, a
// segment starts at a multiple of 32 cells); x lines without explicit part.
template <typename T>
__device__ __forceinline__ void load_seg_x(const T* __restrict__ row, int p, int cnt,
                                           T (&b)[kPSeg - 1]) {
  constexpr int V = 16 / sizeof(T);
#pragma unroll
  for (int q = 0; q < (kPSeg - 1 + V - 1) / V; ++q) {
    if (q * V < cnt) {
      T v[V];
      if constexpr (sizeof(T) == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(row + p) + q);
        v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
      } else {
        const double2 t = __ldg(reinterpret_cast<const double2*>(row + p) + q);
        v[0] = t.x, v[1] = t.y;
      }
#pragma unroll
      for (int e = 0; e < V; ++e)
        if (q * V + e < kPSeg - 1) b[q * V + e] = v[e];
    }
  }
}

template <typename T>
__device__ __forceinline__ T diag_val(const PCoef<T>& k, int i, T b);

// Right-hand side of the K interior cells of a segment starting at p: all
// loads issued before any use (a full segment takes the unguarded path).
template <typename T>
__device__ __forceinline__ void load_interior(const T* __restrict__ row, const PLines& L,
                                              const PCoef<T>& k, int p, int K,
                                              T (&b)[kPSeg - 1]) {
  if (K == kPSeg - 1) {
    if (L.stride == 1 && !k.expl) {
      load_seg_x(row, p, K, b);
    } else {
#pragma unroll
      for (int j = 0; j < kPSeg - 1; ++j) b[j] = rhs_val(row, L, k, p + j);
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < kPSeg - 1; ++j) b[j] = j < K ? rhs_val(row, L, k, p + j) : T(0);
}

template <typename T>
__device__ __forceinline__ T diag_val(const PCoef<T>& k, int i, T b) {
  if (k.dvec) return __ldg(k.dvec + i);
  return k.dbase + k.dc * ((T(4) * b - T(6)) * b + T(2));
}

// Pass 1. Interior cells p .. q-1 (K = len - 1 of them) of segment s, the
// separator q. Record: u_first, u_last, v_first, v_last, w_last, d_q, b_q
// (u: interior solution with zero separators; v / w: response to a unit
// left / right separator; w_first = v_last by symmetry).
template <typename T>
__global__ void __launch_bounds__(kPThreads)
    part_sums(PLines L, PCoef<T> k, const T* __restrict__ in, T* __restrict__ rec) {
  pdl_wait();
  pdl_launch_next();
  int line, s;
  if (!seg_index(L, line, s)) return;
  const T* row = in + line_base(L, line);
  const int p = s * kPSeg;
  const int len = min(kPSeg, L.n - p);
  const int K = len - 1;
  T b[kPSeg - 1];
  load_interior(row, L, k, p, K, b);
  const T a = k.a;
  T uf = 0, ul = 0, vf = 0, vl = 1, wl = 0;  // K = 0: the neighbours are the separators
  if (K > 0) {
    // forward elimination (u, v, w right-hand sides; the last values) and
    // backward elimination from the last interior cell (u, v; the first
    // values), interleaved: two independent chains of pivots; the
    // diagonal is recomputed from b where it is needed
    T cp = 0, yu = 0, yv = 0, yw = 0;
    T cb = 0, zu = 0, zv = 0;
    if (K == kPSeg - 1) {
#pragma unroll
      for (int j = 0; j < kPSeg - 1; ++j) {
        const int jb = kPSeg - 2 - j;  // the same step of the backward chain
        const T inv = rcp(diag_val(k, p + j, b[j]) + a * cp);  // d_j - (-a) c'_{j-1}
        const T invb = rcp(diag_val(k, p + jb, b[jb]) + a * cb);
        yu = (b[j] + a * yu) * inv;
        yv = ((j == 0 ? a : T(0)) + a * yv) * inv;
        yw = ((j == kPSeg - 2 ? a : T(0)) + a * yw) * inv;
        cp = -a * inv;
        zu = (b[jb] + a * zu) * invb;
        zv = ((jb == 0 ? a : T(0)) + a * zv) * invb;
        cb = -a * invb;
      }
    } else {  // the short last segment of a line
#pragma unroll
      for (int j = 0; j < kPSeg - 1; ++j) {
        if (j < K) {
          const T inv = rcp(diag_val(k, p + j, b[j]) + a * cp);
          yu = (b[j] + a * yu) * inv;
          yv = ((j == 0 ? a : T(0)) + a * yv) * inv;
          yw = ((j == K - 1 ? a : T(0)) + a * yw) * inv;
          cp = -a * inv;
        }
      }
#pragma unroll
      for (int j = kPSeg - 2; j >= 0; --j) {
        if (j < K) {
          const T invb = rcp(diag_val(k, p + j, b[j]) + a * cb);
          zu = (b[j] + a * zu) * invb;
          zv = ((j == 0 ? a : T(0)) + a * zv) * invb;
          cb = -a * invb;
        }
      }
    }
    ul = yu;
    vl = yv;
    wl = yw;
    uf = zu;
    vf = zv;
  }
  // the separator's own row (loaded again: a run-time index into b / d
  // would move the arrays to local memory)
  const T bq = rhs_val(row, L, k, p + K);
  const T dq = diag_val(k, p + K, bq);
  T* r = rec + ((int64_t)s * L.nlines + line) * kRec;
  r[0] = uf;
  r[1] = ul;
  r[2] = vf;
  r[3] = vl;
  r[4] = wl;
  r[5] = dq;
  r[6] = bq;
}

// Pass 2, a thread per line: the separators' cyclic tridiagonal system
//   -a v^s_last sep_{s-1} + (d_q - a w^s_last - a v^{s+1}_first) sep_s
//   - a w^{s+1}_first sep_{s+1} = b_q + a (u^s_last + u^{s+1}_first),
// w_first = v_last. Thomas with the Sherman-Morrison correction for the
// corners (m >= 3), a direct solve for m <= 2. Writes sep_s to record slot 7
// and uses slots 5-6 as scratch.
template <typename T, typename Rec>
__device__ __forceinline__ void reduce_line(const Rec& R, int m, T a) {
  // coefficients of separator s (needs records s and s+1)
  auto coef = [&](int s, T& lo, T& di, T& up, T& rhs) {
    const T* r0 = R(s);
    const T* r1 = R(s + 1 == m ? 0 : s + 1);
    lo = -a * r0[3];
    up = -a * r1[3];
    di = r0[5] - a * r0[4] - a * r1[2];
    rhs = r0[6] + a * (r0[1] + r1[0]);
  };
  if (m == 1) {
    T lo, di, up, rhs;
    coef(0, lo, di, up, rhs);
    R(0)[7] = rhs / (di + lo + up);
    return;
  }
  if (m == 2) {
    T l0, d0, u0, r0, l1, d1, u1, r1;
    coef(0, l0, d0, u0, r0);
    coef(1, l1, d1, u1, r1);
    // both neighbours of either separator are the other one
    const T o0 = l0 + u0, o1 = l1 + u1;
    const T det = d0 * d1 - o0 * o1;
    R(0)[7] = (r0 * d1 - o0 * r1) / det;
    R(1)[7] = (d0 * r1 - o1 * r0) / det;
    return;
  }
  // cyclic: row 0 has `lo` at column m-1, row m-1 has `up` at column 0
  T lo0, di0, up0, rh0;
  coef(0, lo0, di0, up0, rh0);
  T loL, diL, upL, rhL;
  coef(m - 1, loL, diL, upL, rhL);
  const T gamma = -di0;
  // forward sweep of T y = rhs and T z = (gamma, 0, ..., 0, upL), with the
  // modified first and last diagonals; records are read kPre at a time so
  // that their loads overlap (the sweep itself is sequential)
  constexpr int kPre = 4;
  T cprev = 0, yprev = 0, zprev = 0;
  for (int s0 = 0; s0 < m; s0 += kPre) {
    T f0[kPre + 1], f2[kPre + 1], f3[kPre + 1], g1[kPre + 1], g4[kPre + 1], g5[kPre + 1],
        g6[kPre + 1];
#pragma unroll
    for (int q = 0; q <= kPre; ++q) {
      const int s = s0 + q;
      if (s <= m) {
        const T* r = R(s == m ? 0 : s);
        f0[q] = r[0], f2[q] = r[2], f3[q] = r[3];
        g1[q] = r[1], g4[q] = r[4], g5[q] = r[5], g6[q] = r[6];
      }
    }
#pragma unroll
    for (int q = 0; q < kPre; ++q) {
      const int s = s0 + q;
      if (s < m) {
        T lo = -a * f3[q];
        T up = -a * f3[q + 1];
        T di = g5[q] - a * g4[q] - a * f2[q + 1];
        const T rh = g6[q] + a * (g1[q] + f0[q + 1]);
        if (s == 0) di = di - gamma;
        if (s == m - 1) di = di - lo0 * upL / gamma;
        const T zr = s == 0 ? gamma : (s == m - 1 ? upL : T(0));
        const T inv = rcp(di - lo * cprev);
        const T c = up * inv;
        const T y = (rh - lo * yprev) * inv;
        const T z = (zr - lo * zprev) * inv;
        T* r = R(s);
        r[5] = c;  // slots 5 (d_q) and 6 (b_q) are no longer needed
        r[6] = y;
        r[7] = z;
        cprev = c, yprev = y, zprev = z;
      }
    }
  }
  // back substitution of both systems
  T ynext = 0, znext = 0, y0 = 0, z0 = 0, yL = 0, zL = 0;
  for (int s1 = m - 1; s1 >= 0; s1 -= kPre) {
    T c5[kPre], c6[kPre], c7[kPre];
#pragma unroll
    for (int q = 0; q < kPre; ++q) {
      const int s = s1 - q;
      if (s >= 0) {
        const T* r = R(s);
        c5[q] = r[5], c6[q] = r[6], c7[q] = r[7];
      }
    }
#pragma unroll
    for (int q = 0; q < kPre; ++q) {
      const int s = s1 - q;
      if (s >= 0) {
        const T y = c6[q] - c5[q] * ynext;
        const T z = c7[q] - c5[q] * znext;
        T* r = R(s);
        r[6] = y;
        r[7] = z;
        if (s == m - 1) yL = y, zL = z;
        if (s == 0) y0 = y, z0 = z;
        ynext = y, znext = z;
      }
    }
  }
  const T fac = (y0 + lo0 * yL / gamma) / (T(1) + z0 + lo0 * zL / gamma);
  for (int s = 0; s < m; ++s) {
    T* r = R(s);
    r[7] = r[6] - fac * r[7];
  }
}

template <typename T>
__global__ void __launch_bounds__(kPThreads)
    part_reduce(PLines L, T a, T* __restrict__ rec) {
  pdl_wait();
  pdl_launch_next();
  const int line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= L.nlines) return;
  reduce_line([&](int s) -> T* { return rec + ((int64_t)s * L.nlines + line) * kRec; },
              L.nseg, a);
}

// The same with a warp's 32 lines staged in shared memory: the records are
// read once, coalesced (each s: 32 consecutive lines), and the sequential
// sweeps run on shared memory (records padded to 9 values: no bank
// conflicts between the lanes). Used while m * 32 * 9 values fit.
constexpr int kRecS = 9;

template <typename T>
__global__ void __launch_bounds__(32)
    part_reduce_smem(PLines L, T a, T* __restrict__ rec) {
  pdl_wait();
  pdl_launch_next();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int lane = threadIdx.x;
  const int line = blockIdx.x * 32 + lane;
  if (line >= L.nlines) return;  // each lane works on its own records only
  const int m = L.nseg;
  for (int s = 0; s < m; ++s) {
    const T* g = rec + ((int64_t)s * L.nlines + line) * kRec;
    T* d = sm + ((int64_t)s * 32 + lane) * kRecS;
#pragma unroll
    for (int k = 0; k < 7; ++k) d[k] = g[k];
  }
  reduce_line([&](int s) -> T* { return sm + ((int64_t)s * 32 + lane) * kRecS; }, m, a);
  for (int s = 0; s < m; ++s)
    rec[((int64_t)s * L.nlines + line) * kRec + 7] = sm[((int64_t)s * 32 + lane) * kRecS + 7];
}

// Pass 3: the interior block with its true separators, then the line.
template <typename T>
__global__ void __launch_bounds__(kPThreads)
    part_solve(PLines L, PCoef<T> k, const T* __restrict__ in, const T* __restrict__ rec,
               T* __restrict__ out) {
  pdl_wait();
  pdl_launch_next();
  int line, s;
  if (!seg_index(L, line, s)) return;
  const int64_t base = line_base(L, line);
  const T* row = in + base;
  const int p = s * kPSeg;
  const int len = min(kPSeg, L.n - p);
  const int K = len - 1;
  const T sep_r = rec[((int64_t)s * L.nlines + line) * kRec + 7];
  const int sl = s == 0 ? L.nseg - 1 : s - 1;
  const T sep_l = rec[((int64_t)sl * L.nlines + line) * kRec + 7];
  T b[kPSeg - 1], d[kPSeg - 1];
  load_interior(row, L, k, p, K, b);
  const T a = k.a;
  // forward elimination, pivots and right-hand sides kept in d and b
  T cp = 0, y = 0;
#pragma unroll 31
  for (int j = 0; j < kPSeg - 1; ++j) {
    if (j < K) {
      const T rj = b[j] + (j == 0 ? a * sep_l : T(0)) + (j == K - 1 ? a * sep_r : T(0));
      const T inv = rcp(diag_val(k, p + j, b[j]) + a * cp);
      y = (rj + a * y) * inv;
      cp = -a * inv;
      d[j] = cp;
      b[j] = y;
    }
  }
  T* orow = out + base;
  T x = 0;
#pragma unroll 31
  for (int j = kPSeg - 2; j >= 0; --j) {
    if (j < K) {
      x = j == K - 1 ? b[j] : b[j] - d[j] * x;
      orow[(int64_t)(p + j) * L.stride] = x;
    }
  }
  orow[(int64_t)(p + K) * L.stride] = sep_r;
}

PLines make_plines(const Geo& g, int axis) {
  const int nz = g.ndim == 3 ? g.n[0] : 1, ny = g.n[g.ndim - 2], nx = g.n[g.ndim - 1];
  const int64_t plane = g.ndim == 3 ? g.plane : (int64_t)g.pitch * ny;
  const int p = axis + (3 - g.ndim);  // 0 z, 1 y, 2 x
  PLines L{};
  L.pitch = g.pitch;
  L.plane = plane;
  L.nx = nx;
  L.ny = ny;
  if (p == 2) {
    L.n = nx;
    L.stride = 1;
    L.xfast = 0;
    L.nlines = ny * nz;
  } else {
    L.xfast = 1;
    L.n = p == 1 ? ny : nz;
    L.stride = p == 1 ? g.pitch : plane;
    L.no = p == 1 ? nz : ny;
    L.ostride = p == 1 ? plane : g.pitch;
    L.nlines = nx * L.no;
  }
  L.nseg = (L.n + kPSeg - 1) / kPSeg;
  return L;
}

size_t part_scratch_bytes(const Geo& g, int axis, int eb) {
  const PLines L = make_plines(g, axis);
  return (size_t)L.nlines * L.nseg * kRec * eb;
}

// Variable-diagonal periodic line solve along `axis` (C order).
template <typename T>
int32_t var_sweep(const Geo& g, int axis, double a, double dbase, double dc, const T* dvec,
                  int expl, double ea, const T* in, T* out, void* scratch, size_t bytes,
                  cudaStream_t st) {
  if (axis < 0 || axis >= g.ndim) return fail(PPF_ERR_INVALID, "axis %d out of range", axis);
  if (!(a > 0) || !isfinite(a) || !isfinite(dbase) || !isfinite(dc) || !isfinite(ea))
    return fail(PPF_ERR_INVALID, "alpha must be finite and > 0");
  const PLines L = make_plines(g, axis);
  if (L.n < 3)
    return fail(PPF_ERR_INVALID, "periodic line solves need >= 3 cells along the axis (got %d)",
                L.n);
  if (expl && in == out)
    return fail(PPF_ERR_INVALID, "in and out must differ when an explicit part is folded in");
  const size_t need = part_scratch_bytes(g, axis, sizeof(T));
  if (!scratch || bytes < need)
    return fail(PPF_ERR_INVALID, "scratch of %zu bytes needed (got %zu)", need, bytes);
  PCoef<T> k{};
  k.a = (T)a;
  k.dbase = (T)dbase;
  k.dc = (T)dc;
  k.expl = expl;
  k.w0 = (T)(1.0 - 2.0 * ea);
  k.w1 = (T)ea;
  k.dvec = dvec;
  T* rec = static_cast<T*>(scratch);
  const int64_t threads = (int64_t)L.nlines * L.nseg;
  const dim3 grid((unsigned)((threads + kPThreads - 1) / kPThreads));
  PPF_TRY_CUDA(launch(part_sums<T>, grid, dim3(kPThreads), 0, st, true, L, k, in, rec));
  // one warp per block: the lines' sequential sweeps spread over every SM
  const size_t sm_bytes = (size_t)L.nseg * 32 * kRecS * sizeof(T);
  if (sm_bytes <= 200 * 1024) {
    static bool attr_set[2] = {false, false};
    if (!attr_set[sizeof(T) == 8]) {
      PPF_TRY_CUDA(allow_smem(part_reduce_smem<T>, 200 * 1024));
      attr_set[sizeof(T) == 8] = true;
    }
    PPF_TRY_CUDA(launch(part_reduce_smem<T>, dim3((L.nlines + 31) / 32), dim3(32), sm_bytes, st,
                        true, L, (T)a, rec));
  } else {
    PPF_TRY_CUDA(launch(part_reduce<T>, dim3((L.nlines + 31) / 32), dim3(32), 0, st, true, L,
                        (T)a, rec));
  }
  PPF_TRY_CUDA(launch(part_solve<T>, grid, dim3(kPThreads), 0, st, true, L, k, in,
                      (const T*)rec, out));
  return PPF_OK;
}

// ---------------------------------------------------------------- pointwise
// dvec[i] = dbase + dc (4 phi^2 - 6 phi + 2) at the i-th cell of the C-order
// flattened interior (CahnAllen.py:228-235: np.fill_diagonal takes the
// first n entries of the flattened 3-D source term).
template <typename T>
__global__ void flat_diag(Geo g, const T* __restrict__ phi, int n, T dbase, T dc, T* dvec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nx = g.n[g.ndim - 1], ny = g.n[g.ndim - 2];
  const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
  const T v = phi[(int64_t)z * g.plane + (int64_t)y * g.pitch + x];
  dvec[i] = dbase + dc * ((T(4) * v - T(6)) * v + T(2));
}

// IMEX right-hand side phi - c (4 phi^3 - 6 phi^2 - 2 phi) (CahnAllen.py:264,
// its -2 phi as written), 1-D row.
template <typename T>
__global__ void imex_rhs(const T* __restrict__ in, T* __restrict__ out, int n, T c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T v = in[i];
  out[i] = v - c * (((T(4) * v - T(6)) * v - T(2)) * v);
}

// Cahn-Hilliard explicit part of the 1-D Crank-Nicolson engine
// (CahnHilliard.py:186-193): mu = -eps^2 lap(c) + 4c^3 - 6c^2 + 2c, then
// c + M lap(mu) (no dt, as written), periodic.
template <typename T>
__global__ void ch_mu(const T* __restrict__ c, T* __restrict__ mu, int n, T e2idx2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T v = c[i], l = c[i == 0 ? n - 1 : i - 1], r = c[i == n - 1 ? 0 : i + 1];
  mu[i] = -e2idx2 * (l + r - T(2) * v) + ((T(4) * v - T(6)) * v + T(2)) * v;
}

template <typename T>
__global__ void ch_apply(const T* __restrict__ c, const T* __restrict__ mu, T* __restrict__ out,
                         int n, T Midx2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T m0 = mu[i], l = mu[i == 0 ? n - 1 : i - 1], r = mu[i == n - 1 ? 0 : i + 1];
  out[i] = c[i] + Midx2 * (l + r - T(2) * m0);
}

// ---------------------------------------------------------------- 1-D CH
// One cyclic pentadiagonal system (engine_CahnHilliardImplicit1D,
// CahnHilliard.py:148-163): row j has 1 + a (2 s_j + 6 e) on the diagonal,
// -a (s_j + 4 e) at j -/+ 1, a e at j -/+ 2, s = 4c^2 - 6c + 2, e =
// eps^2 / dx^2, a = M dt / dx^2. One thread: banded elimination without
// pivoting of the non-periodic part B, five right-hand sides (c and the
// unit vectors at rows 0, 1, n-2, n-1), and the Woodbury correction
// x = y - Z (I + V^T Z)^-1 V^T y for the six corner entries. Work space
// (n >= 5 cells): 10 n values of T.
template <typename T>
__global__ void ch_penta(const T* __restrict__ c, T* __restrict__ out, int n, T a, T e,
                         T* __restrict__ w) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  // band storage of row j: lo2, lo1, di, up1, up2 in w[5j .. 5j+4]
  T* band = w;
  T* rhs = w + 5 * (int64_t)n;  // 5 right-hand sides, column-major [5][n]
  for (int j = 0; j < n; ++j) {
    const T v = c[j];
    const T s = (T(4) * v - T(6)) * v + T(2);
    band[5 * j + 0] = a * e;
    band[5 * j + 1] = -a * (s + T(4) * e);
    band[5 * j + 2] = T(1) + a * (T(2) * s + T(6) * e);
    band[5 * j + 3] = -a * (s + T(4) * e);
    band[5 * j + 4] = a * e;
    rhs[j] = v;
    for (int q = 1; q < 5; ++q) rhs[(int64_t)q * n + j] = T(0);
  }
  // corner entries (row, column, value), E = U V^T with U = unit rows
  const int crow[4] = {0, 1, n - 2, n - 1};
  // V^T rows: row 0: (n-2: lo2_0), (n-1: lo1_0); row 1: (n-1: lo2_1);
  // row n-2: (0: up2_{n-2}); row n-1: (0: up1_{n-1}), (1: up2_{n-1})
  const T v00 = band[0], v01 = band[1], v1 = band[5 * 1 + 0];
  const T v2 = band[5 * (n - 2) + 4], v30 = band[5 * (n - 1) + 3], v31 = band[5 * (n - 1) + 4];
  for (int q = 0; q < 4; ++q) rhs[(int64_t)(q + 1) * n + crow[q]] = T(1);
  // elimination (no pivoting) of the band, applied to the five columns
  for (int j = 0; j < n; ++j) {
    const T piv = band[5 * j + 2];
    for (int r = 1; r <= 2 && j + r < n; ++r) {
      const T f = band[5 * (j + r) + 2 - r] / piv;  // entry (j + r, j)
      band[5 * (j + r) + 2 - r] = T(0);
      // row j + r -= f * row j over columns j+1 .. j+2
      band[5 * (j + r) + 3 - r] -= f * band[5 * j + 3];
      if (j + 2 < n) band[5 * (j + r) + 4 - r] -= f * band[5 * j + 4];
      for (int q = 0; q < 5; ++q)
        rhs[(int64_t)q * n + j + r] -= f * rhs[(int64_t)q * n + j];
    }
  }
  for (int q = 0; q < 5; ++q) {
    T* x = rhs + (int64_t)q * n;
    for (int j = n - 1; j >= 0; --j) {
      T v = x[j];
      if (j + 1 < n) v -= band[5 * j + 3] * x[j + 1];
      if (j + 2 < n) v -= band[5 * j + 4] * x[j + 2];
      x[j] = v / band[5 * j + 2];
    }
  }
  // V^T applied to a column
  auto vt = [&](const T* x, int r) -> T {
    if (r == 0) return v00 * x[n - 2] + v01 * x[n - 1];
    if (r == 1) return v1 * x[n - 1];
    if (r == 2) return v2 * x[0];
    return v30 * x[0] + v31 * x[1];
  };
  T S[4][5];  // [I + V^T Z | V^T y]
  for (int r = 0; r < 4; ++r) {
    for (int q = 0; q < 4; ++q) S[r][q] = (r == q ? T(1) : T(0)) + vt(rhs + (int64_t)(q + 1) * n, r);
    S[r][4] = vt(rhs, r);
  }
  for (int i = 0; i < 4; ++i) {  // Gaussian elimination with partial pivoting, 4 x 4
    int pr = i;
    for (int r = i + 1; r < 4; ++r)
      if (fabs((double)S[r][i]) > fabs((double)S[pr][i])) pr = r;
    if (pr != i)
      for (int q = 0; q < 5; ++q) {
        const T t = S[i][q];
        S[i][q] = S[pr][q];
        S[pr][q] = t;
      }
    for (int r = i + 1; r < 4; ++r) {
      const T f = S[r][i] / S[i][i];
      for (int q = i; q < 5; ++q) S[r][q] -= f * S[i][q];
    }
  }
  T wv[4];
  for (int i = 3; i >= 0; --i) {
    T v = S[i][4];
    for (int q = i + 1; q < 4; ++q) v -= S[i][q] * wv[q];
    wv[i] = v / S[i][i];
  }
  for (int j = 0; j < n; ++j) {
    T v = rhs[j];
    for (int q = 0; q < 4; ++q) v -= rhs[(int64_t)(q + 1) * n + j] * wv[q];
    out[j] = v;
  }
}

// ---------------------------------------------------------------- full 2-D
// Chebyshev with Jacobi scaling for (1 + 4a + c g(phi)) x - a sum(nbrs) =
// phi (engine_CahnAllenImplicit2D_GMRES, CahnAllen.py:163-175): the scaled
// operator's spectrum lies in [1 - rho, 1 + rho], rho = 4a / d_min,
// d_min = 1 + 4a - c / 4 (g's minimum is -1/4).
template <typename T>
__global__ void __launch_bounds__(256)
    jacobi_cheb(Geo g, T dbase, T dc, T a, T omega, int first, const T* __restrict__ b,
                const T* __restrict__ y, const T* yprev, T* ynew) {
  pdl_wait();
  pdl_launch_next();
  const int nx = g.n[1], ny = g.n[0];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
  for (int yy = blockIdx.y; yy < ny; yy += gridDim.y) {
    const int64_t ym = (int64_t)(yy == 0 ? ny - 1 : yy - 1) * g.pitch;
    const int64_t yp = (int64_t)(yy == ny - 1 ? 0 : yy + 1) * g.pitch;
    const int64_t yb = (int64_t)yy * g.pitch;
    const int64_t i = yb + x;
    const T bv = __ldg(b + i);
    const T d = dbase + dc * ((T(4) * bv - T(6)) * bv + T(2));
    const T yc = __ldg(y + i);
    const T sy = __ldg(y + yb + xm) + __ldg(y + yb + xp) + __ldg(y + ym + x) + __ldg(y + yp + x);
    const T rich = yc + (bv - (d * yc - a * sy)) / d;
    ynew[i] = first ? rich : yprev[i] + omega * (rich - yprev[i]);
  }
}

template <typename T>
int32_t jacobi_solve(const Geo& g, double a, double dbase, double dc, double tol, const T* in,
                     T* out, T* tmp, int32_t* iterations, cudaStream_t st) {
  if (dc < 0) return fail(PPF_ERR_UNSUPPORTED, "the full system needs M W dt >= 0");
  const double dmin = dbase - 0.25 * dc;
  const double rho = 4.0 * a / dmin;
  if (!(dmin > 0) || !(rho < 1))
    return fail(PPF_ERR_UNSUPPORTED,
                "the full implicit system is not diagonally dominant for this dt "
                "(16 W M dt / 4 >= 1): the Chebyshev bound does not hold");
  if (!tmp || tmp == in || tmp == out)
    return fail(PPF_ERR_INVALID, "the full solve needs a tmp field distinct from in and out");
  const double need = 2.0 * (1.0 + rho) / (1.0 - rho) / tol;
  int iters = rho > 0 ? (int)ceil(acosh(need) / acosh(1.0 / rho)) : 1;
  if (iters < 1) iters = 1;
  if (iterations) *iterations = iters;
  const dim3 grid((g.n[1] + 255) / 256, (unsigned)(g.n[0] < 65535 ? g.n[0] : 65535));
  const T* prev = nullptr;
  const T* cur = in;
  double om = 1.0;
  const double rho2 = rho * rho;
  for (int j = 1; j <= iters; ++j) {
    if (j == 2)
      om = 2.0 / (2.0 - rho2);
    else if (j > 2)
      om = 1.0 / (1.0 - rho2 * om / 4.0);
    T* dst = ((iters - j) % 2 == 0) ? out : tmp;
    PPF_TRY_CUDA(launch(jacobi_cheb<T>, grid, dim3(256), 0, st, true, g, (T)dbase, (T)dc, (T)a,
                        (T)om, j == 1 ? 1 : 0, in, cur, prev, dst));
    prev = cur;
    cur = dst;
  }
  return PPF_OK;
}

// ---------------------------------------------------------------- MINRES
// The same full 2-D system where the Chebyshev bound fails (16 W M dt >= 4:
// the diagonal 1 + 4a + c g(phi) can fall below the off-diagonal sum and
// the symmetric matrix may be indefinite; the reference's GMRES still
// returns a step). MINRES (Paige & Saunders 1975, in the Lanczos form of
// Elman, Silvester & Wathen, Algorithm 2.4) solves symmetric indefinite
// systems with short recurrences: one matrix-vector product and two inner
// products per iteration. It runs as ONE persistent cooperative kernel:
// every CTA resident, the iterations separated by grid barriers (three per
// iteration: after the product and its inner product, after the Lanczos
// vector and its norm, after the solution update), the inner products
// accumulated in double from per-CTA partial sums that every CTA adds up in
// the same order (so every CTA takes the same scalars and the same stopping
// decision). The loop ends on the device when the residual norm (|eta|,
// exact in exact arithmetic) reaches tol ||b||, when the Lanczos process
// finds an invariant subspace (solved), or, unconverged, after max_iter
// iterations or at a singular tridiagonal (both set
// PPF_STATUS_NOT_CONVERGED). Initial guess: b (the field before the step).
constexpr int kMinresThreads = 256;
constexpr int kMinresMaxCtas = 2048;
constexpr int kMinresMaxIter = 20000;

struct MinresBufs {
  void* v0;  // Lanczos vector v_{j-1}
  void* v1;  // v_j
  void* t;   // A v_j, then the next Lanczos vector before its scaling
  void* w0;  // w_{j-2}
  void* w1;  // w_{j-1}
  double* part_a;  // per-CTA partial sums (two arrays: consecutive reductions)
  double* part_b;
  unsigned* sync;  // grid barrier words
  int* info;       // [0] iterations run, [1] converged
};

__device__ __forceinline__ double block_sum_d(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < kMinresThreads / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) red[0] = r;
  }
  __syncthreads();
  r = red[0];
  __syncthreads();
  return r;
}

// Sum of the n partials, in the same order in every CTA.
__device__ __forceinline__ double total(const double* part, int n, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += kMinresThreads) v += part[i];
  return block_sum_d(v, red);
}

template <typename T>
__global__ void __launch_bounds__(kMinresThreads)
    minres_kernel(Geo g, T dbase, T dc, T a, double tol, int max_iter, const T* __restrict__ b,
                  T* __restrict__ x, MinresBufs bufs, int* status) {
  __shared__ double red[kMinresThreads / 32];
  __shared__ int flag;
  if (threadIdx.x == 0) flag = 0;
  const int nx = g.n[1], ny = g.n[0];
  const int nb = gridDim.x;
  T* V0 = (T*)bufs.v0;
  T* V1 = (T*)bufs.v1;
  T* Tv = (T*)bufs.t;
  T* W0 = (T*)bufs.w0;
  T* W1 = (T*)bufs.w1;
  // (A y)_i = d_i y_i - a (sum of the four periodic neighbours),
  // d_i = dbase + dc g(b_i): the reference's matrix (CahnAllen.py:170-176)
  auto apply = [&](const T* y, int row, int col) -> T {
    const int64_t yb = (int64_t)row * g.pitch;
    const int64_t ym = (int64_t)(row == 0 ? ny - 1 : row - 1) * g.pitch;
    const int64_t yp = (int64_t)(row == ny - 1 ? 0 : row + 1) * g.pitch;
    const int xm = col == 0 ? nx - 1 : col - 1, xp = col == nx - 1 ? 0 : col + 1;
    const T bv = b[yb + col];
    const T d = dbase + dc * ((T(4) * bv - T(6)) * bv + T(2));
    const T sy = (y[yb + xm] + y[yb + xp]) + (y[ym + col] + y[yp + col]);
    return d * y[yb + col] - a * sy;
  };
#define PPF_CELLS                                                   \
  for (int row = blockIdx.x; row < ny; row += nb)                   \
    for (int col = threadIdx.x; col < nx; col += kMinresThreads)
#define PPF_SYNC \
  if (!grid_barrier(bufs.sync, nb, status, &flag)) return

  // r0 = b - A b into V1, x = b, w = 0; ||r0||^2 and ||b||^2
  double pr = 0.0, pb = 0.0;
  PPF_CELLS {
    const int64_t i = (int64_t)row * g.pitch + col;
    const T bv = b[i];
    const T r = bv - apply(b, row, col);
    V1[i] = r;
    x[i] = bv;
    V0[i] = T(0);
    W0[i] = T(0);
    W1[i] = T(0);
    pr += (double)r * (double)r;
    pb += (double)bv * (double)bv;
  }
  pr = block_sum_d(pr, red);
  pb = block_sum_d(pb, red);
  if (threadIdx.x == 0) {
    bufs.part_a[blockIdx.x] = pr;
    bufs.part_b[blockIdx.x] = pb;
  }
  PPF_SYNC;
  const double beta1 = sqrt(total(bufs.part_a, nb, red));
  const double bnorm = sqrt(total(bufs.part_b, nb, red));
  const double goal = tol * bnorm;
  int it = 0;
  bool converged = beta1 <= goal;
  if (!converged) {
    const T inv = (T)(1.0 / beta1);
    PPF_CELLS {
      const int64_t i = (int64_t)row * g.pitch + col;
      V1[i] *= inv;
    }
    PPF_SYNC;
    double beta = beta1, eta = beta1;
    double c_prev = 1.0, c = 1.0, s_prev = 0.0, sg = 0.0;
    for (it = 1; it <= max_iter; ++it) {
      // t = A v_j; alpha = v_j . A v_j
      double pa = 0.0;
      PPF_CELLS {
        const int64_t i = (int64_t)row * g.pitch + col;
        const T av = apply(V1, row, col);
        Tv[i] = av;
        pa += (double)V1[i] * (double)av;
      }
      pa = block_sum_d(pa, red);
      if (threadIdx.x == 0) bufs.part_a[blockIdx.x] = pa;
      PPF_SYNC;
      const double alpha = total(bufs.part_a, nb, red);
      // t = A v_j - alpha v_j - beta v_{j-1}; its norm
      double pn = 0.0;
      PPF_CELLS {
        const int64_t i = (int64_t)row * g.pitch + col;
        const T tv = Tv[i] - (T)alpha * V1[i] - (T)beta * V0[i];
        Tv[i] = tv;
        pn += (double)tv * (double)tv;
      }
      pn = block_sum_d(pn, red);
      if (threadIdx.x == 0) bufs.part_b[blockIdx.x] = pn;
      PPF_SYNC;
      const double beta_n = sqrt(total(bufs.part_b, nb, red));
      // Givens rotations of the tridiagonal's QR factorisation
      const double a0 = c * alpha - c_prev * sg * beta;
      const double a1 = sqrt(a0 * a0 + beta_n * beta_n);
      if (!(a1 > 0.0) || !isfinite(a1) || !isfinite(alpha)) break;  // singular: not converged
      const double a2 = sg * alpha + c_prev * c * beta;
      const double a3 = s_prev * beta;
      const double c_n = a0 / a1, s_n = beta_n / a1;
      const double step = c_n * eta;
      const T inv_b = beta_n > 0 ? (T)(1.0 / beta_n) : T(0);
      // v_{j+1} = t / beta_n into V0; w_j = (v_j - a3 w_{j-2} - a2 w_{j-1}) / a1
      // into W0; x += c_n eta w_j
      PPF_CELLS {
        const int64_t i = (int64_t)row * g.pitch + col;
        const T w = (V1[i] - (T)a3 * W0[i] - (T)a2 * W1[i]) / (T)a1;
        W0[i] = w;
        x[i] += (T)step * w;
        V0[i] = Tv[i] * inv_b;
      }
      eta = -s_n * eta;
      c_prev = c;
      c = c_n;
      s_prev = sg;
      sg = s_n;
      beta = beta_n;
      T* tmp = V0;
      V0 = V1;
      V1 = tmp;  // v_j becomes v_{j-1}, v_{j+1} becomes v_j
      tmp = W0;
      W0 = W1;
      W1 = tmp;  // w_j is now the newest
      if (fabs(eta) <= goal || beta_n == 0.0) {
        converged = true;
        break;
      }
      PPF_SYNC;
    }
  }
#undef PPF_CELLS
#undef PPF_SYNC
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    bufs.info[0] = it;
    bufs.info[1] = converged ? 1 : 0;
    if (!converged) atomicOr(status, PPF_STATUS_NOT_CONVERGED);
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t minres_scratch_bytes(const Geo& g, int eb) {
  const size_t vec = align256((size_t)g.n[0] * g.pitch * eb);
  return 5 * vec + 2 * align256(kMinresMaxCtas * sizeof(double)) + 256;
}

template <typename T>
int32_t minres_solve(const Geo& g, double a, double dbase, double dc, double tol, int max_iter,
                     const T* in, T* out, void* scratch, size_t bytes, int32_t* iterations,
                     cudaStream_t st) {
  if (bytes < minres_scratch_bytes(g, sizeof(T)))
    return fail(PPF_ERR_INVALID, "the MINRES solve needs %zu bytes of scratch",
                minres_scratch_bytes(g, sizeof(T)));
  int* status = status_ptr();
  if (!status) return fail(PPF_ERR_CUDA, "status word unavailable");
  char* p = static_cast<char*>(scratch);
  const size_t vec = align256((size_t)g.n[0] * g.pitch * sizeof(T));
  MinresBufs bb;
  bb.v0 = p;
  bb.v1 = p + vec;
  bb.t = p + 2 * vec;
  bb.w0 = p + 3 * vec;
  bb.w1 = p + 4 * vec;
  bb.part_a = reinterpret_cast<double*>(p + 5 * vec);
  bb.part_b = reinterpret_cast<double*>(p + 5 * vec + align256(kMinresMaxCtas * sizeof(double)));
  char* tail = p + 5 * vec + 2 * align256(kMinresMaxCtas * sizeof(double));
  bb.sync = reinterpret_cast<unsigned*>(tail);
  bb.info = reinterpret_cast<int*>(tail + 16);
  PPF_TRY_CUDA(cudaMemsetAsync(tail, 0, 256, st));
  auto kern = minres_kernel<T>;
  int dev = 0, sms = 0, per_sm = 0;
  PPF_TRY_CUDA(cudaGetDevice(&dev));
  PPF_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PPF_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMinresThreads, 0));
  long long ctas = (long long)sms * (per_sm < 1 ? 1 : per_sm);
  if (ctas > kMinresMaxCtas) ctas = kMinresMaxCtas;
  if (ctas > g.n[0]) ctas = g.n[0];
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(kMinresThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PPF_TRY_CUDA(cudaLaunchKernelEx(&cfg, kern, g, (T)dbase, (T)dc, (T)a, tol, max_iter, in, out,
                                  bb, status));
  if (iterations) *iterations = -max_iter;  // run on the device: at most max_iter
  return PPF_OK;
}

// ---------------------------------------------------------------- dispatch

size_t phase_scratch_bytes(const Geo& g, int eb) {
  size_t m = 0;
  for (int ax = 0; ax < g.ndim; ++ax) {
    const size_t b = part_scratch_bytes(g, ax, eb);
    m = b > m ? b : m;
  }
  const bool oned = g.ndim == 2 && g.n[0] == 1;
  const size_t dv = (size_t)(g.n[0] + g.n[1] + g.n[2]) * eb;
  const size_t penta = oned ? (size_t)10 * g.n[1] * eb : 0;
  const size_t base = align256(m) + align256(dv) + align256(penta);
  // the full 2-D solve beyond the Chebyshev bound (MINRES) reuses the same
  // scratch from its start
  const size_t mr = (g.ndim == 2 && !oned) ? minres_scratch_bytes(g, eb) : 0;
  return base > mr ? base : mr;
}

template <typename T>
int32_t copy_field(const Geo& g, const T* in, T* out, cudaStream_t st) {
  const int64_t rows = g.ndim == 3 ? (int64_t)g.n[0] * g.n[1] : g.n[0];
  PPF_TRY_CUDA(cudaMemcpyAsync(out, in, (size_t)rows * g.pitch * sizeof(T),
                               cudaMemcpyDeviceToDevice, st));
  return PPF_OK;
}

template <typename T>
int32_t phase_step(const PpfImplicitPhaseParams* p, const PpfGrid* grid, const T* in, T* out,
                   T* tmp, void* scratch, size_t bytes, int32_t* iterations, void* stream) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out || in == out) return fail(PPF_ERR_INVALID, "in and out must be distinct");
  if (!(p->dx > 0) || !(p->dt >= 0) || !isfinite(p->M) || !isfinite(p->W) ||
      !isfinite(p->epsilon) || !isfinite(p->dt))
    return fail(PPF_ERR_INVALID, "dx > 0, dt >= 0 and finite M, W, epsilon are required");
  if (p->model != PPF_MODEL_ALLEN_CAHN && p->model != PPF_MODEL_CAHN_HILLIARD)
    return fail(PPF_ERR_INVALID, "model must be PPF_MODEL_ALLEN_CAHN or PPF_MODEL_CAHN_HILLIARD");
  if (p->solver != PPF_SOLVER_IMPLICIT && p->solver != PPF_SOLVER_CRANK_NICOLSON &&
      p->solver != PPF_SOLVER_IMEX)
    return fail(PPF_ERR_INVALID, "solver must be implicit, Crank-Nicolson or IMEX");
  const size_t need = phase_scratch_bytes(g, sizeof(T));
  if (!scratch || bytes < need)
    return fail(PPF_ERR_INVALID, "scratch of %zu bytes needed (got %zu)", need, bytes);
  for (int ax = 0; ax < g.ndim; ++ax)
    if (g.n[ax] < 3 && !(ax == 0 && g.ndim == 2 && g.n[0] == 1))
      return fail(PPF_ERR_INVALID, "implicit solves need >= 3 cells per axis (axis %d has %d)",
                  ax, g.n[ax]);
  cudaStream_t st = (cudaStream_t)stream;
  if (iterations) *iterations = 0;
  const bool oned = g.ndim == 2 && g.n[0] == 1;
  const int dims = oned ? 1 : g.ndim;
  const double dx2 = p->dx * p->dx;
  const double a = p->M * p->dt * p->epsilon * p->epsilon / dx2;
  const double wm = p->W * p->M * p->dt;
  char* sc = static_cast<char*>(scratch);
  size_t recb = 0;
  for (int ax = 0; ax < g.ndim; ++ax) {
    const size_t b = part_scratch_bytes(g, ax, sizeof(T));
    recb = b > recb ? b : recb;
  }
  T* dvec = reinterpret_cast<T*>(sc + align256(recb));
  T* work = reinterpret_cast<T*>(sc + align256(recb) +
                                 align256((size_t)(g.n[0] + g.n[1] + g.n[2]) * sizeof(T)));
  const int n1 = g.n[1];
  const int nb = (n1 + 255) / 256;
  if (p->model == PPF_MODEL_CAHN_HILLIARD && oned && p->solver != PPF_SOLVER_IMEX) {
    if (n1 < 5) return fail(PPF_ERR_INVALID, "the 1-D Cahn-Hilliard solve needs >= 5 cells");
    const double e = p->epsilon * p->epsilon / dx2;
    double h = p->dt;
    const T* src = in;
    if (p->solver == PPF_SOLVER_CRANK_NICOLSON) {
      if (!tmp || tmp == in || tmp == out)
        return fail(PPF_ERR_INVALID, "Crank-Nicolson needs a tmp field distinct from in and out");
      h = p->dt / 2;
      ch_mu<T><<<nb, 256, 0, st>>>(in, work, n1, (T)e);
      PPF_TRY_CUDA(cudaGetLastError());
      ch_apply<T><<<nb, 256, 0, st>>>(in, work, tmp, n1, (T)(p->M / dx2));
      PPF_TRY_CUDA(cudaGetLastError());
      src = tmp;
    }
    ch_penta<T><<<1, 32, 0, st>>>(src, out, n1, (T)(p->M * h / dx2), (T)e, work);
    PPF_TRY_CUDA(cudaGetLastError());
    return PPF_OK;
  }
  // Allen-Cahn (and the Cahn-Hilliard engines that copy its formulas)
  if (p->solver == PPF_SOLVER_IMEX) {
    if (dims != 1) return copy_field(g, in, out, st);  // "not yet implemented": unchanged
    if (!tmp || tmp == in || tmp == out)
      return fail(PPF_ERR_INVALID, "IMEX needs a tmp field distinct from in and out");
    imex_rhs<T><<<nb, 256, 0, st>>>(in, tmp, n1, (T)(16.0 * wm));
    PPF_TRY_CUDA(cudaGetLastError());
    if constexpr (sizeof(T) == 4)
      return ppf_line_solve_f32(grid, 1, a, -1, 0.0, tmp, out, scratch, bytes, stream);
    else
      return ppf_line_solve_f64(grid, 1, a, -1, 0.0, tmp, out, scratch, bytes, stream);
  }
  if (p->solver == PPF_SOLVER_CRANK_NICOLSON) {
    if (dims != 2) return copy_field(g, in, out, st);  // the reference returns unchanged
    if (!tmp || tmp == in || tmp == out)
      return fail(PPF_ERR_INVALID, "Crank-Nicolson needs a tmp field distinct from in and out");
    const double h = 0.5 * a;
    rc = var_sweep<T>(g, 1, h, 1 + 2 * h, 8 * wm, nullptr, 1, h, in, tmp, scratch, bytes, st);
    if (rc) return rc;
    return var_sweep<T>(g, 0, h, 1 + 2 * h, 8 * wm, nullptr, 1, h, tmp, out, scratch, bytes, st);
  }
  // implicit
  if (dims == 1) return var_sweep<T>(g, 1, a, 1 + 2 * a, 16 * wm, nullptr, 0, 0.0, in, out,
                                     scratch, bytes, st);
  if (dims == 2) {
    if (p->gmres && !p->adi) {
      const double dbase = 1 + 4 * a, dc = 16 * wm;
      const double dmin = dbase - 0.25 * dc;
      if (dc >= 0 && dmin > 0 && 4.0 * a / dmin < 1) {
        const double tol = p->tol > 0 ? p->tol : (sizeof(T) == 4 ? 1e-7 : 1e-14);
        return jacobi_solve<T>(g, a, dbase, dc, tol, in, out, tmp, iterations, st);
      }
      const double tol = p->tol > 0 ? p->tol : (sizeof(T) == 4 ? 1e-7 : 1e-14);
      if (p->max_iter < 0) return fail(PPF_ERR_INVALID, "max_iter must be >= 0");
      return minres_solve<T>(g, a, dbase, dc, tol, p->max_iter ? p->max_iter : kMinresMaxIter,
                             in, out, scratch, bytes, iterations, st);
    }
    rc = var_sweep<T>(g, 1, a, 1 + 2 * a, 8 * wm, nullptr, 0, 0.0, in, out, scratch, bytes, st);
    if (rc) return rc;
    return var_sweep<T>(g, 0, a, 1 + 2 * a, 8 * wm, nullptr, 0, 0.0, out, out, scratch, bytes,
                        st);
  }
  // 3-D: one shared diagonal per axis from the flattened source term of the
  // field before the step
  T* dv[3] = {dvec, dvec + g.n[0], dvec + g.n[0] + g.n[1]};
  for (int ax = 0; ax < 3; ++ax) {
    flat_diag<T><<<(g.n[ax] + 255) / 256, 256, 0, st>>>(g, in, g.n[ax], (T)(1 + 2 * a),
                                                        (T)(16 * wm / 3), dv[ax]);
    PPF_TRY_CUDA(cudaGetLastError());
  }
  const T* src = in;
  for (int ax = 2; ax >= 0; --ax) {
    rc = var_sweep<T>(g, ax, a, 0.0, 0.0, dv[ax], 0, 0.0, src, out, scratch, bytes, st);
    if (rc) return rc;
    src = out;
  }
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_phase_implicit_scratch_bytes(const PpfGrid* grid, int32_t elem_bytes,
                                         size_t* bytes) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!bytes) return fail(PPF_ERR_INVALID, "bytes is NULL");
  if (elem_bytes != 4 && elem_bytes != 8) return fail(PPF_ERR_INVALID, "elem_bytes must be 4 or 8");
  size_t line = 0;
  rc = ppf_implicit_scratch_bytes(grid, elem_bytes, &line);
  if (rc) return rc;
  const size_t b = phase_scratch_bytes(g, elem_bytes);
  *bytes = b > line ? b : line;
  return PPF_OK;
}

int32_t ppf_var_line_solve_f32(const PpfGrid* grid, int32_t axis, double alpha, double dbase,
                               double dcoef, const float* dvec, int32_t expl, double expl_alpha,
                               const float* in, float* out, void* scratch,
                               size_t scratch_bytes, void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  return var_sweep<float>(g, axis, alpha, dbase, dcoef, dvec, expl ? 1 : 0, expl_alpha, in, out,
                          scratch, scratch_bytes, (cudaStream_t)stream);
}

int32_t ppf_var_line_solve_f64(const PpfGrid* grid, int32_t axis, double alpha, double dbase,
                               double dcoef, const double* dvec, int32_t expl,
                               double expl_alpha, const double* in, double* out, void* scratch,
                               size_t scratch_bytes, void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!in || !out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  return var_sweep<double>(g, axis, alpha, dbase, dcoef, dvec, expl ? 1 : 0, expl_alpha, in,
                           out, scratch, scratch_bytes, (cudaStream_t)stream);
}

int32_t ppf_phase_implicit_step_f32(const PpfImplicitPhaseParams* p, const PpfGrid* g,
                                    const float* in, float* out, float* tmp, void* scratch,
                                    size_t scratch_bytes, int32_t* iterations, void* stream) {
  return phase_step<float>(p, g, in, out, tmp, scratch, scratch_bytes, iterations, stream);
}

int32_t ppf_phase_implicit_step_f64(const PpfImplicitPhaseParams* p, const PpfGrid* g,
                                    const double* in, double* out, double* tmp, void* scratch,
                                    size_t scratch_bytes, int32_t* iterations, void* stream) {
  return phase_step<double>(p, g, in, out, tmp, scratch, scratch_bytes, iterations, stream);
}

}  // extern "C"
