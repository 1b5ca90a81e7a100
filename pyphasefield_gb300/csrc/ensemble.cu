// Batched ensemble: many Warren1995 and Allen-Cahn instances with uneven 2-D
// grids and per-instance parameters advanced one step by ONE persistent
// launch.
//
// Work items are warp bands (a 30-column strip x ROWS rows of one member);
// member m owns items [item_begin[m], item_begin[m+1]). A persistent grid of
// warps walks the items round-robin (every warp gets the same count, +-1),
// finds each item's member by binary search over item_begin, and runs that
// member's band update (w95_core.cuh for Warren1995, the Allen-Cahn band
// below). Each member has its own ping-pong buffers; `parity` selects the
// direction, so a captured graph of an even number of steps replays
// unchanged.
//
// Reference: engine_Warren1995 (Engines/Warren1995.py:50-92) and
// engine_CahnAllenExplicit (Engines/CahnAllen.py:128-135), one instance per
// Simulation in the reference.
#include <string.h>

#include <vector>

#include "ppf_common.cuh"
#include "w95_core.cuh"

namespace ppf {
namespace {

constexpr int kWarpsPerCta = 4;
constexpr int kCtaThreads = 32 * kWarpsPerCta;

struct MemberDev {
  int model;
  int strips;
  long long item_begin;
  Geo g;
  Bc<float> bc;
  float* phi[2];
  float* c[2];
  unsigned long long seed;
  w95::Coef<float> w;
  float ac_a, ac_b;  // dt M eps^2 / dx^2, dt M 16 W
};

// Allen-Cahn band in the warp-strip layout: phi + a lap - b (4phi^3 - 6phi^2
// + 2phi), neighbour sum grouped ((w + e) + (n + s)) as in the single-grid
// kernel.
template <int ROWS>
__device__ __forceinline__ void ac_band(float a, float b, const Geo& g, const Bc<float>& bc,
                                        const float* __restrict__ in, float* __restrict__ out,
                                        int xs, int y0) {
  const int lane = threadIdx.x;
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + lane;
  const bool x_in = xs >= 0 && xs + 31 < nx;
  const bool owner = lane >= 1 && lane <= w95::kStrip && x < nx;
  float v[ROWS + 2];
#pragma unroll
  for (int j = 0; j < ROWS + 2; ++j) {
    const int row = y0 - 1 + j;
    v[j] = (x_in && (unsigned)row < (unsigned)ny) ? __ldg(in + (int64_t)row * g.pitch + x)
                                                   : fetch<float, 2>(in, g, bc, 0, row, x);
  }
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

template <int ROWS>
__global__ void __launch_bounds__(kCtaThreads, 8)
    ensemble_kernel(const MemberDev* __restrict__ members, int n_members, long long n_items,
                    int parity, uint64_t step, const uint64_t* __restrict__ step_base) {
  const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
  long long it = (long long)blockIdx.x * kWarpsPerCta + threadIdx.y;
  if (it >= n_items) return;  // whole warp
  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;
  for (; it < n_items; it += nwarps) {
    int lo = 0, hi = n_members - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (members[mid].item_begin <= it) lo = mid;
      else hi = mid - 1;
    }
    const MemberDev& m = members[lo];
    const int local = (int)(it - m.item_begin);
    const int xs = (local % m.strips) * w95::kStrip - 1;
    const int y0 = (local / m.strips) * ROWS;
    // the member's constants are copied to registers once per item: the
    // band reads them many times, and from global memory each read would be
    // a dependent load
    const Geo g = m.g;
    const Bc<float> bc = m.bc;
    if (m.model == PPF_MODEL_WARREN1995) {
      const w95::Coef<float> k = m.w;
      w95::band<float, ROWS>(k, g, bc, m.phi[parity], m.c[parity], m.phi[1 - parity],
                             m.c[1 - parity], m.seed, step, xs, y0);
    } else {
      ac_band<ROWS>(m.ac_a, m.ac_b, g, bc, m.phi[parity], m.phi[1 - parity], xs, y0);
    }
  }
}

int32_t build_table(const PpfMember* members, int32_t n, const PpfTiling* tiling,
                    std::vector<MemberDev>* out, long long* n_items, int* rows) {
  if (!members || n < 1 || n > (1 << 20))
    return fail(PPF_ERR_INVALID, "ensemble needs 1..2^20 members (got %d)", n);
  *rows = tiling && tiling->tile_y ? tiling->tile_y : 2;
  if (*rows != 2 && *rows != 4 && *rows != 8)
    return fail(PPF_ERR_INVALID, "ensemble rows per warp must be 2, 4 or 8");
  if (tiling && tiling->depth > 1)
    return fail(PPF_ERR_UNSUPPORTED, "ensemble steps advance one step per pass");
  const bool bulk = !(tiling && (tiling->flags & PPF_TILING_FULL_EVAL));
  out->resize(n);
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
    d.item_begin = items;
    items += (long long)d.strips * ((s.ny + *rows - 1) / *rows);
  }
  *n_items = items;
  return PPF_OK;
}

template <int ROWS>
cudaError_t launch_ensemble(const PpfEnsemblePlan* p, int parity, uint64_t step,
                            const uint64_t* step_base, bool pdl, cudaStream_t s) {
  auto kern = ensemble_kernel<ROWS>;
  static int sms = 0, per_sm = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCtaThreads, 0) !=
            cudaSuccess || per_sm < 1)
      per_sm = 1;
  }
  // fewest warps that still give every warp the same item count (+-1)
  const long long resident = (long long)sms * per_sm * kWarpsPerCta;
  const long long rounds = (p->n_items + resident - 1) / resident;
  const long long warps = (p->n_items + rounds - 1) / rounds;
  const long long ctas = (warps + kWarpsPerCta - 1) / kWarpsPerCta;
  return launch(kern, dim3((unsigned)ctas), dim3(32, kWarpsPerCta), 0, s, pdl,
                (const MemberDev*)p->device_table, p->n_members, (long long)p->n_items, parity,
                step, step_base);
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
  long long items;
  int rows;
  int32_t rc = build_table(members, n, tiling, &t, &items, &rows);
  if (rc) return rc;
  *bytes = t.size() * sizeof(MemberDev);
  return PPF_OK;
}

int32_t ppf_ensemble_build(const PpfMember* members, int32_t n, const PpfTiling* tiling,
                           void* device_table, size_t bytes, PpfEnsemblePlan* plan,
                           void* stream) {
  clear_error();
  if (!device_table || !plan) return fail(PPF_ERR_INVALID, "NULL table or plan");
  std::vector<MemberDev> t;
  long long items;
  int rows;
  int32_t rc = build_table(members, n, tiling, &t, &items, &rows);
  if (rc) return rc;
  if (bytes < t.size() * sizeof(MemberDev))
    return fail(PPF_ERR_INVALID, "table needs %zu bytes, got %zu", t.size() * sizeof(MemberDev),
                bytes);
  if (((uintptr_t)device_table) % 16) return fail(PPF_ERR_INVALID, "table not 16-byte aligned");
  if (items > (1LL << 40)) return fail(PPF_ERR_INVALID, "ensemble too large");
  cudaStream_t s = (cudaStream_t)stream;
  PPF_TRY_CUDA(cudaMemcpyAsync(device_table, t.data(), t.size() * sizeof(MemberDev),
                               cudaMemcpyHostToDevice, s));
  PPF_TRY_CUDA(cudaStreamSynchronize(s));  // the host table dies with this call
  plan->device_table = device_table;
  plan->n_items = items;
  plan->n_members = n;
  plan->rows = rows;
  return PPF_OK;
}

int32_t ppf_ensemble_step_f32(const PpfEnsemblePlan* plan, int32_t parity, uint64_t step,
                              const uint64_t* step_base, const PpfTiling* tiling, void* stream) {
  clear_error();
  if (!plan || !plan->device_table) return fail(PPF_ERR_INVALID, "plan is NULL");
  if (parity != 0 && parity != 1) return fail(PPF_ERR_INVALID, "parity must be 0 or 1");
  if (plan->n_items < 1) return fail(PPF_ERR_INVALID, "empty plan");
  const bool pdl = tiling && tiling->pdl;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  switch (plan->rows) {
    case 2: e = launch_ensemble<2>(plan, parity, step, step_base, pdl, s); break;
    case 4: e = launch_ensemble<4>(plan, parity, step, step_base, pdl, s); break;
    case 8: e = launch_ensemble<8>(plan, parity, step, step_base, pdl, s); break;
    default: return fail(PPF_ERR_INVALID, "plan rows %d invalid", plan->rows);
  }
  if (e != cudaSuccess) return fail(PPF_ERR_CUDA, "ensemble launch: %s", cudaGetErrorString(e));
  return PPF_OK;
}

}  // extern "C"
