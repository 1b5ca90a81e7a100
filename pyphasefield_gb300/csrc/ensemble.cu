// Batched ensemble: many Warren1995 and Allen-Cahn instances with uneven 2-D
// grids and per-instance parameters, advanced together.
//
// Work: a member's grid is cut into warp bands (a 30-column strip x ROWS
// rows), and its bands are grouped 4 x BANDS at a time into units, one per
// CTA (BANDS per warp); a member's last unit is padded so that no unit spans
// two members. A unit table maps every unit to its member, so a CTA finds
// its member with one load and stages the member's folded constants in
// shared memory for its four warps.
//
// Two-row tilings: ensemble_f2_kernel, one plain launch per step over every
// unit (the single-grid float kernel's band code and register budget); four-
// and eight-row tilings run without a grid-barrier buffer the same way
// (ensemble_tall_kernel). Four- and eight-row tilings given one:
// ensemble_kernel, one cooperative, persistent launch per chunk of steps
// (same results bit for bit): each CTA walks the units grid-stride, then all
// CTAs meet at a grid barrier before the next step (each member's ping-pong
// buffers swap by step parity). The barrier's waits are bounded: a CTA that
// waits too long sets PPF_STATUS_TIMEOUT and the launch ends early. Reads of
// the fields use plain (coherent) loads there, since other CTAs of the same
// launch wrote them.
//
// Reference: engine_Warren1995 (Engines/Warren1995.py:50-92) and
// engine_CahnAllenExplicit (Engines/CahnAllen.py:128-135), one instance per
// Simulation in the reference.
#include <string.h>

#include <vector>

#include "ppf_common.cuh"
#include "ppf_grid.cuh"
#include "w95_core.cuh"

namespace ppf {
namespace {

constexpr int kWarpsPerCta = 4;
constexpr int kCtaThreads = 32 * kWarpsPerCta;

struct MemberDev {
  int model;
  int strips;
  unsigned long long strips_magic;  // ceil(2^64 / strips): band / strips by one multiply
  long long item_begin;  // first band (items of a member are [begin, begin + items))
  long long items;
  long long unit_begin;  // first unit
  Geo g;
  Bc<float> bc;
  float* phi[2];
  float* c[2];
  unsigned long long seed;
  w95::Coef<float> w;
  float ac_a, ac_b;  // dt M eps^2 / dx^2, dt M 16 W
};

// Device table layout: MemberDev[n_members], then int unit_member[n_units].
inline size_t units_offset(int n) { return ((size_t)n * sizeof(MemberDev) + 15) / 16 * 16; }

// Band b of a member (b < 2^32) as strip and row band: b / strips through the
// member's 64-bit reciprocal (exact for 32-bit dividends: the error of the
// rounded-up reciprocal, b / 2^64, stays below 1 / strips), instead of a
// 64-bit division.
__device__ __forceinline__ void band_coords(const MemberDev& m, unsigned b, int& strip,
                                            int& rowband) {
  const unsigned q = m.strips == 1 ? b : (unsigned)__umul64hi((unsigned long long)b, m.strips_magic);
  rowband = (int)q;
  strip = (int)(b - q * (unsigned)m.strips);
}

// Allen-Cahn band in the warp-strip layout: phi + a lap - b (4phi^3 - 6phi^2
// + 2phi), neighbour sum grouped ((w + e) + (n + s)) as in the single-grid
// kernel. ac_load requests rows y0 - 1 .. y0 + ROWS of this lane's column
// (straight from one base pointer for an interior band, from the lane's
// source column when only the x edge is crossed), ac_compute writes rows
// y0 .. y0 + ROWS - 1.
template <int ROWS, bool COHERENT>
__device__ __forceinline__ void ac_load(const Geo& g, const Bc<float>& bc,
                                        const float* __restrict__ in, int xs, int y0,
                                        float (&v)[ROWS + 2]) {
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + (int)threadIdx.x;
  if (xs >= 0 && xs + 32 <= nx && y0 >= 1 && y0 + ROWS + 1 <= ny) {  // warp-uniform
    const float* p = in + (int64_t)(y0 - 1) * g.pitch + x;
#pragma unroll
    for (int j = 0; j < ROWS + 2; ++j) v[j] = ldf<COHERENT>(p + (int64_t)j * g.pitch);
    return;
  }
  if (y0 >= 1 && y0 + ROWS + 1 <= ny) {  // rows inside, strip across the x edge
    const ColumnRule<float, 1> cr(g, bc, x);
    const float* p = in + (int64_t)(y0 - 1) * g.pitch + cr.xi;
#pragma unroll
    for (int j = 0; j < ROWS + 2; ++j) v[j] = ldf<COHERENT>(p + (int64_t)j * g.pitch);
#pragma unroll
    for (int j = 0; j < ROWS + 2; ++j) v[j] = cr.value(0, v[j]);
    return;
  }
  const bool x_in = (unsigned)x < (unsigned)nx;
#pragma unroll
  for (int j = 0; j < ROWS + 2; ++j) {
    const int row = y0 - 1 + j;
    v[j] = (x_in && (unsigned)row < (unsigned)ny)
               ? ldf<COHERENT>(in + (int64_t)row * g.pitch + x)
               : fetch<float, 2, COHERENT>(in, g, bc, 0, row, x);
  }
}

template <int ROWS>
__device__ __forceinline__ void ac_compute(float a, float b, const Geo& g,
                                           float* __restrict__ out, int xs, int y0,
                                           const float (&v)[ROWS + 2]) {
  const int lane = threadIdx.x;
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + lane;
  const bool owner = lane >= 1 && lane <= w95::kStrip && x < nx;
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const float c = v[r + 1];
    const float w = w95::shfl_w(c), e = w95::shfl_e(c);
    const float lap = ((w + e) + (v[r] + v[r + 2])) - 4.0f * c;
    const float fp = c * (2.0f + c * (-6.0f + 4.0f * c));
    const int row = y0 + r;
    if (owner && row < ny) out[(int64_t)row * g.pitch + x] = c + (a * lap - b * fp);
  }
}

template <int ROWS, bool COHERENT>
__device__ __forceinline__ void ac_band(float a, float b, const Geo& g, const Bc<float>& bc,
                                        const float* __restrict__ in, float* __restrict__ out,
                                        int xs, int y0) {
  float v[ROWS + 2];
  ac_load<ROWS, COHERENT>(g, bc, in, xs, y0, v);
  ac_compute<ROWS>(a, b, g, out, xs, y0, v);
}

// A unit is BANDS bands per warp; warp w of the CTA takes bands w, w + 4,
// ... of the unit's 4 BANDS (the CTA's warps work on neighbouring strips at
// any moment).
// Warren1995 members: the next band's rows are requested before the current
// band is computed, so a warp's loads overlap its own arithmetic.
template <int ROWS, int BANDS>
__device__ __forceinline__ void run_unit(const MemberDev& m, long long unit, int parity,
                                         uint64_t step) {
  const long long first = (unit - m.unit_begin) * (kWarpsPerCta * BANDS);
  if (m.model == PPF_MODEL_WARREN1995) {
    long long local = first + threadIdx.y;
    if (local >= m.items) return;  // whole warp
    float bp[ROWS + 2], bcv[ROWS + 2];
    int strip, rowband;
    band_coords(m, (unsigned)local, strip, rowband);
    int xs = strip * w95::kStrip - 1;
    int y0 = rowband * ROWS;
    w95::band_load<float, ROWS, true>(m.g, m.bc, m.phi[parity], m.c[parity], xs, y0, bp, bcv);
#pragma unroll 1
    for (int j = 0; j < BANDS; ++j) {
      const long long nxt = local + kWarpsPerCta;
      const bool more = j + 1 < BANDS && nxt < m.items;
      float np[ROWS + 2], ncv[ROWS + 2];
      int nxs = 0, ny0 = 0;
      if (more) {
        band_coords(m, (unsigned)nxt, strip, rowband);
        nxs = strip * w95::kStrip - 1;
        ny0 = rowband * ROWS;
        w95::band_load<float, ROWS, true>(m.g, m.bc, m.phi[parity], m.c[parity], nxs, ny0, np,
                                          ncv);
      }
      w95::band_compute<float, ROWS>(m.w, m.g, m.phi[1 - parity], m.c[1 - parity], m.seed,
                                     step, xs, y0, bp, bcv);
      if (!more) return;
#pragma unroll
      for (int r = 0; r < ROWS + 2; ++r) {
        bp[r] = np[r];
        bcv[r] = ncv[r];
      }
      local = nxt;
      xs = nxs;
      y0 = ny0;
    }
    return;
  }
#pragma unroll 1
  for (int j = 0; j < BANDS; ++j) {
    const long long local = first + j * kWarpsPerCta + threadIdx.y;
    if (local >= m.items) return;  // past the member's last band (whole warp)
    int strip, rowband;
    band_coords(m, (unsigned)local, strip, rowband);
    const int xs = strip * w95::kStrip - 1;
    const int y0 = rowband * ROWS;
    ac_band<ROWS, true>(m.ac_a, m.ac_b, m.g, m.bc, m.phi[parity], m.phi[1 - parity], xs, y0);
  }
}

// Resident CTAs per SM asked of the register allocator for the persistent
// kernel: the member's constants come from shared memory into registers and
// the next band is prefetched, so a band of two or four rows needs up to
// 126 registers a thread and eight rows 151 without spills.
template <int ROWS>
struct EnsMinBlocks {
  static constexpr int value = ROWS <= 4 ? 4 : 3;
};

template <int ROWS, int BANDS>
__global__ void __launch_bounds__(kCtaThreads, (EnsMinBlocks<ROWS>::value))
    ensemble_kernel(const MemberDev* __restrict__ members, const int* __restrict__ unit_member,
                    long long n_units, int parity, uint64_t step,
                    const uint64_t* __restrict__ step_base, int nsteps, unsigned* sync,
                    int* status) {
  __shared__ MemberDev sm;
  __shared__ int flag;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  if (tid == 0) flag = 0;
  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;
  for (int s = 0; s < nsteps; ++s) {
    const int par = (parity + s) & 1;
    for (long long u = blockIdx.x; u < n_units; u += gridDim.x) {
      const int mi = unit_member[u];
      __syncthreads();  // the previous unit is done with sm
      {
        const int* src = reinterpret_cast<const int*>(members + mi);
        int* dst = reinterpret_cast<int*>(&sm);
        for (int i = tid; i < (int)(sizeof(MemberDev) / 4); i += kCtaThreads) dst[i] = src[i];
      }
      __syncthreads();
      run_unit<ROWS, BANDS>(sm, u, par, step + s);
    }
    if (s + 1 < nsteps && !grid_barrier(sync, gridDim.x, status, &flag)) return;
  }
}

// One step over every unit, one CTA per unit (4 BANDS bands of one member;
// warp w takes bands w, w + 4, ...): the ensemble counterpart of the
// single-grid float kernels (warren1995.cu). A plain launch per step (no grid
// barrier). The member's record is staged in shared memory once per CTA,
// before waiting on the previous step (the plan table is written before the
// first launch and never by a step, so with programmatic dependent launch
// these loads overlap that step's tail), and a band's strip and row band come
// from the member's reciprocal of its strip count. A Warren1995 band that
// takes the full update draws its own Philox blocks: members early in a run
// are mostly bulk, and a bulk band draws none.
template <int ROWS, int BANDS>
__device__ __forceinline__ void step_units(const MemberDev* __restrict__ members,
                                           const int* __restrict__ unit_member, int parity,
                                           uint64_t step, const uint64_t* __restrict__ step_base,
                                           MemberDev& m) {
  const int w = threadIdx.y;
  const int tid = threadIdx.x + 32 * w;
  {
    const int* src = reinterpret_cast<const int*>(members + unit_member[blockIdx.x]);
    int* dst = reinterpret_cast<int*>(&m);
    for (int i = tid; i < (int)(sizeof(MemberDev) / 4); i += kCtaThreads) dst[i] = src[i];
  }
  __syncthreads();
  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;
  // the member's bands are < 2^32 (checked when the plan is built)
  const unsigned first = (blockIdx.x - (unsigned)m.unit_begin) * (kWarpsPerCta * BANDS);
  const unsigned items = (unsigned)m.items;
  const bool warren = m.model == PPF_MODEL_WARREN1995;
#pragma unroll 1
  for (int j = 0; j < BANDS; ++j) {
    const unsigned local = first + (unsigned)(w + kWarpsPerCta * j);
    if (local >= items) return;  // whole warp
    int strip, rowband;
    band_coords(m, local, strip, rowband);
    const int xs = strip * w95::kStrip - 1;
    const int y0 = rowband * ROWS;
    if (!warren) {
      ac_band<ROWS, false>(m.ac_a, m.ac_b, m.g, m.bc, m.phi[parity], m.phi[1 - parity], xs, y0);
      continue;
    }
    float bp[ROWS + 2], bcv[ROWS + 2];
    w95::band_load<float, ROWS>(m.g, m.bc, m.phi[parity], m.c[parity], xs, y0, bp, bcv);
    w95::band_compute_pk<ROWS / 2>(m.w, m.g, m.phi[1 - parity], m.c[1 - parity], m.seed, step,
                                   xs, y0, bp, bcv);
  }
}

// Two-row bands: twelve CTAs per SM (40 registers a thread with a few
// spilled: measured faster than ten CTAs without spills).
template <int BANDS>
__global__ void __launch_bounds__(kCtaThreads, 12)
    ensemble_f2_kernel(const MemberDev* __restrict__ members,
                       const int* __restrict__ unit_member, int parity, uint64_t step,
                       const uint64_t* __restrict__ step_base) {
  __shared__ MemberDev m;
  step_units<2, BANDS>(members, unit_member, parity, step, step_base, m);
}

// Four- and eight-row bands stepped the same way (plans of those heights run
// without a grid-barrier buffer): eight CTAs per SM at four rows (64
// registers), six at eight rows (80).
template <int ROWS, int BANDS>
__global__ void __launch_bounds__(kCtaThreads, ROWS == 4 ? 8 : 6)
    ensemble_tall_kernel(const MemberDev* __restrict__ members,
                         const int* __restrict__ unit_member, int parity, uint64_t step,
                         const uint64_t* __restrict__ step_base) {
  __shared__ MemberDev m;
  step_units<ROWS, BANDS>(members, unit_member, parity, step, step_base, m);
}

int32_t build_table(const PpfMember* members, int32_t n, const PpfTiling* tiling,
                    std::vector<MemberDev>* out, std::vector<int>* units, long long* n_items,
                    int* rows, int* bands) {
  if (!members || n < 1 || n > (1 << 20))
    return fail(PPF_ERR_INVALID, "ensemble needs 1..2^20 members (got %d)", n);
  *rows = tiling && tiling->tile_y ? tiling->tile_y : 2;
  if (*rows != 2 && *rows != 4 && *rows != 8)
    return fail(PPF_ERR_INVALID, "ensemble rows per warp must be 2, 4 or 8");
  *bands = tiling && tiling->tile_x ? tiling->tile_x : 4;
  if (*bands != 1 && *bands != 4 && !(*rows == 2 && (*bands == 8 || *bands == 16)))
    return fail(PPF_ERR_INVALID,
                "ensemble bands per warp (tile_x) must be 1 or 4 (or 8, 16 with two rows)");
  if (tiling && tiling->depth > 1)
    return fail(PPF_ERR_UNSUPPORTED, "ensemble steps advance one step per pass");
  const bool bulk = !(tiling && (tiling->flags & PPF_TILING_FULL_EVAL));
  out->resize(n);
  units->clear();
  long long items = 0;
  for (int i = 0; i < n; ++i) {
    const PpfMember& s = members[i];
    MemberDev& d = (*out)[i];
    memset(&d, 0, sizeof(d));
    if (s.model != PPF_MODEL_WARREN1995 && s.model != PPF_MODEL_ALLEN_CAHN)
      return fail(PPF_ERR_INVALID, "member %d: unknown model %d", i, s.model);
    PpfGrid pg{};
    pg.ndim = 2;
    pg.shape[0] = s.ny;
    pg.shape[1] = s.nx;
    pg.pitch = s.pitch;
    int32_t rc = make_geo(&pg, 2, 2, &d.g);
    if (rc) return fail(rc, "member %d: bad grid", i);
    const bool w95m = s.model == PPF_MODEL_WARREN1995;
    const double dx = w95m ? s.w95.dx : s.ac.dx;
    if (!(dx > 0)) return fail(PPF_ERR_INVALID, "member %d: dx must be > 0", i);
    if ((rc = make_bc<float>(&s.bc, d.g, dx, w95m ? 2 : 1, 1, &d.bc)))
      return fail(rc, "member %d: bad boundary", i);
    if (!s.phi[0] || !s.phi[1] || s.phi[0] == s.phi[1] ||
        (w95m && (!s.c[0] || !s.c[1] || s.c[0] == s.c[1])))
      return fail(PPF_ERR_INVALID, "member %d: buffers missing or aliased", i);
    d.model = s.model;
    d.phi[0] = s.phi[0];
    d.phi[1] = s.phi[1];
    d.c[0] = s.c[0];
    d.c[1] = s.c[1];
    d.seed = s.seed;
    if (w95m) {
      if (!(s.w95.T > 0) || !(s.w95.T_mA > 0) || !(s.w95.T_mB > 0) || !(s.w95.R > 0))
        return fail(PPF_ERR_INVALID, "member %d: T, T_mA, T_mB and R must be > 0", i);
      d.w = w95::fold<float>(s.w95, bulk);
    } else {
      d.ac_a = (float)(s.ac.dt * s.ac.M * s.ac.epsilon * s.ac.epsilon / (dx * dx));
      d.ac_b = (float)(s.ac.dt * s.ac.M * 16.0 * s.ac.W);
    }
    d.strips = (int)((s.nx + w95::kStrip - 1) / w95::kStrip);
    d.strips_magic = d.strips > 1 ? ~0ULL / (unsigned long long)d.strips + 1 : 0;
    d.item_begin = items;
    d.items = (long long)d.strips * ((s.ny + *rows - 1) / *rows);
    if (d.items >= (1LL << 32)) return fail(PPF_ERR_INVALID, "member %d: too many bands", i);
    d.unit_begin = (long long)units->size();
    const long long per_unit = (long long)kWarpsPerCta * *bands;
    const long long nu = (d.items + per_unit - 1) / per_unit;
    if ((long long)units->size() + nu > (1LL << 31) - 1)
      return fail(PPF_ERR_INVALID, "ensemble too large");
    units->insert(units->end(), (size_t)nu, i);
    items += d.items;
  }
  *n_items = items;
  return PPF_OK;
}

struct Occupancy {
  int sms = 0, per_sm = 0;
};

template <int ROWS, int BANDS>
cudaError_t launch_ensemble(const PpfEnsemblePlan* p, int parity, uint64_t step,
                            const uint64_t* step_base, int nsteps, unsigned* sync, int* status,
                            bool pdl, cudaStream_t s) {
  auto kern = ensemble_kernel<ROWS, BANDS>;
  static Occupancy occ[SymbolCache::kMaxDevices];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= SymbolCache::kMaxDevices) return cudaErrorInvalidDevice;
  Occupancy& o = occ[dev];
  if (!o.sms) {
    int sms = 0, per_sm = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCtaThreads, 0)) !=
        cudaSuccess)
      return e;
    o.per_sm = per_sm < 1 ? 1 : per_sm;
    o.sms = sms;
  }
  const char* base = reinterpret_cast<const char*>(p->device_table);
  const MemberDev* members = reinterpret_cast<const MemberDev*>(base);
  const int* units = reinterpret_cast<const int*>(base + units_offset(p->n_members));
  // every CTA resident (cooperative), each walking the same number of
  // units (+-1)
  const long long resident = (long long)o.sms * o.per_sm;
  const long long rounds = (p->n_units + resident - 1) / resident;
  const long long ctas = (p->n_units + rounds - 1) / rounds;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(32, kWarpsPerCta);
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  int na = 0;
  if (nsteps > 1) {
    attr[na].id = cudaLaunchAttributeCooperative;
    attr[na].val.cooperative = 1;
    ++na;
  } else if (pdl) {
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  return cudaLaunchKernelEx(&cfg, kern, members, units, (long long)p->n_units, parity, step,
                            step_base, nsteps, sync, status);
}

// nsteps launches of a per-step kernel (ensemble_f2_kernel or
// ensemble_tall_kernel), each over every unit.
template <typename Kernel>
cudaError_t launch_plain_steps(Kernel kern, const PpfEnsemblePlan* p, int parity, uint64_t step,
                               const uint64_t* step_base, int nsteps, bool pdl, cudaStream_t s) {
  if (p->n_units > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const char* base = reinterpret_cast<const char*>(p->device_table);
  const MemberDev* members = reinterpret_cast<const MemberDev*>(base);
  const int* units = reinterpret_cast<const int*>(base + units_offset(p->n_members));
  for (int i = 0; i < nsteps; ++i) {
    const cudaError_t e =
        launch(kern, dim3((unsigned)p->n_units), dim3(32, kWarpsPerCta), 0, s, pdl, members,
               units, (parity + i) & 1, step + (uint64_t)i, step_base);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int32_t run(const PpfEnsemblePlan* plan, int32_t parity, uint64_t step,
            const uint64_t* step_base, int32_t nsteps, void* sync, const PpfTiling* tiling,
            void* stream) {
  if (!plan || !plan->device_table) return fail(PPF_ERR_INVALID, "plan is NULL");
  if (parity != 0 && parity != 1) return fail(PPF_ERR_INVALID, "parity must be 0 or 1");
  if (plan->n_items < 1 || plan->n_units < 1) return fail(PPF_ERR_INVALID, "empty plan");
  if (nsteps < 1) return fail(PPF_ERR_INVALID, "nsteps must be >= 1");
  if (plan->rows != 2 && sync && ((uintptr_t)sync) % 8)
    return fail(PPF_ERR_INVALID, "the grid-barrier sync buffer must be 8-byte aligned");
  int* status = status_ptr();
  if (!status) return fail(PPF_ERR_CUDA, "status word unavailable");
  const bool pdl = tiling && tiling->pdl;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* sy = (unsigned*)sync;
  cudaError_t e;
#define PPF_ENS(R, B) launch_ensemble<R, B>(plan, parity, step, step_base, nsteps, sy, status, pdl, s)
#define PPF_PLAIN(K) launch_plain_steps(K, plan, parity, step, step_base, nsteps, pdl, s)
  // four- and eight-row plans: the persistent kernel when given a barrier
  // buffer, per-step launches without one
  const int key = plan->rows * 100 + plan->bands + (plan->rows != 2 && sy ? 10000 : 0);
  switch (key) {
    case 201: e = PPF_PLAIN(ensemble_f2_kernel<1>); break;
    case 204: e = PPF_PLAIN(ensemble_f2_kernel<4>); break;
    case 208: e = PPF_PLAIN(ensemble_f2_kernel<8>); break;
    case 216: e = PPF_PLAIN(ensemble_f2_kernel<16>); break;
    case 401: e = PPF_PLAIN((ensemble_tall_kernel<4, 1>)); break;
    case 404: e = PPF_PLAIN((ensemble_tall_kernel<4, 4>)); break;
    case 801: e = PPF_PLAIN((ensemble_tall_kernel<8, 1>)); break;
    case 804: e = PPF_PLAIN((ensemble_tall_kernel<8, 4>)); break;
    case 10401: e = PPF_ENS(4, 1); break;
    case 10404: e = PPF_ENS(4, 4); break;
    case 10801: e = PPF_ENS(8, 1); break;
    case 10804: e = PPF_ENS(8, 4); break;
    default: return fail(PPF_ERR_INVALID, "plan rows %d / bands %d invalid", plan->rows,
                         plan->bands);
  }
#undef PPF_PLAIN
#undef PPF_ENS
  if (e != cudaSuccess) return fail(PPF_ERR_CUDA, "ensemble launch: %s", cudaGetErrorString(e));
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_ensemble_plan_bytes(const PpfMember* members, int32_t n, const PpfTiling* tiling,
                                size_t* bytes) {
  clear_error();
  if (!bytes) return fail(PPF_ERR_INVALID, "bytes is NULL");
  std::vector<MemberDev> t;
  std::vector<int> units;
  long long items;
  int rows, bands;
  int32_t rc = build_table(members, n, tiling, &t, &units, &items, &rows, &bands);
  if (rc) return rc;
  *bytes = units_offset(n) + units.size() * sizeof(int);
  return PPF_OK;
}

int32_t ppf_ensemble_build(const PpfMember* members, int32_t n, const PpfTiling* tiling,
                           void* device_table, size_t bytes, PpfEnsemblePlan* plan,
                           void* stream) {
  clear_error();
  if (!device_table || !plan) return fail(PPF_ERR_INVALID, "NULL table or plan");
  std::vector<MemberDev> t;
  std::vector<int> units;
  long long items;
  int rows, bands;
  int32_t rc = build_table(members, n, tiling, &t, &units, &items, &rows, &bands);
  if (rc) return rc;
  const size_t need = units_offset(n) + units.size() * sizeof(int);
  if (bytes < need) return fail(PPF_ERR_INVALID, "table needs %zu bytes, got %zu", need, bytes);
  if (((uintptr_t)device_table) % 16) return fail(PPF_ERR_INVALID, "table not 16-byte aligned");
  if (items > (1LL << 40)) return fail(PPF_ERR_INVALID, "ensemble too large");
  std::vector<unsigned char> host(need, 0);
  memcpy(host.data(), t.data(), t.size() * sizeof(MemberDev));
  memcpy(host.data() + units_offset(n), units.data(), units.size() * sizeof(int));
  cudaStream_t s = (cudaStream_t)stream;
  PPF_TRY_CUDA(cudaMemcpyAsync(device_table, host.data(), need, cudaMemcpyHostToDevice, s));
  PPF_TRY_CUDA(cudaStreamSynchronize(s));  // the host table dies with this call
  plan->device_table = device_table;
  plan->n_items = items;
  plan->n_members = n;
  plan->rows = rows;
  plan->bands = bands;
  plan->reserved = 0;
  plan->n_units = (int64_t)units.size();
  return PPF_OK;
}

int32_t ppf_ensemble_step_f32(const PpfEnsemblePlan* plan, int32_t parity, uint64_t step,
                              const uint64_t* step_base, const PpfTiling* tiling, void* stream) {
  clear_error();
  return run(plan, parity, step, step_base, 1, nullptr, tiling, stream);
}

int32_t ppf_ensemble_run_f32(const PpfEnsemblePlan* plan, int32_t parity, uint64_t step,
                             const uint64_t* step_base, int32_t nsteps, void* sync,
                             const PpfTiling* tiling, void* stream) {
  clear_error();
  return run(plan, parity, step, step_base, nsteps, sync, tiling, stream);
}

}  // extern "C"
