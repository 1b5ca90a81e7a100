// Warren-Boettinger (1995) band update for float with packed FP32x2
// arithmetic (add/sub/mul/fma.rn.f32x2): two neighbouring output rows travel
// as the two halves of one 64-bit register pair, so every arithmetic
// instruction of the update advances both rows. Same equations
// and cell layout as the scalar band in w95_core.cuh (Engines/Warren1995.py
// :50-92); the exact bulk form and the noise stream are unchanged.
#pragma once

#include <cstdint>

namespace ppf {
namespace w95 {

struct F2 {
  uint64_t v;
};

__device__ __forceinline__ F2 pk(float a, float b) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ F2 sp(float a) { return pk(a, a); }
__device__ __forceinline__ float lo(F2 x) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
  return a;
}
__device__ __forceinline__ float hi(F2 x) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
  return b;
}
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// a * b + c, one rounding per half
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// D~ and Q~ (see point() in w95_core.cuh) for two cells at once.
__device__ __forceinline__ void point2(const Coef<float>& k, F2 phi, F2 c, F2& Dt, F2& Qt) {
  const F2 one = sp(1.f);
  const F2 p = phi * phi * phi * fma2(phi, fma2(sp(6.f), phi, sp(-15.f)), sp(10.f));
  const F2 om = one - phi;
  const F2 g = phi * phi * (om * om);
  const F2 gp = phi * fma2(phi, fma2(sp(4.f), phi, sp(-6.f)), sp(2.f));
  Dt = fma2(sp(k.a1), p, sp(k.a0));
  const F2 dH = fma2(sp(k.WB - k.WA), gp, sp(k.hB - k.hA) * g);
  Qt = Dt * sp(k.vr) * c * (one - c) * dH;
}

template <typename T>
__device__ __forceinline__ T shfl_w(T v);
template <typename T>
__device__ __forceinline__ T shfl_e(T v);

// Exact bulk test of a band (see band_compute in w95_core.cuh): every lane's
// R2 loaded rows (the owned cells' 3x3 neighbourhoods and a little more) hold
// one value v, exactly 0 or 1. Then D~ is uniform and equals
// a0 + a1 p(v) = fma(a1, v, a0) bit for bit (p(0) = 0, p(1) = 1 exactly),
// Q~ and every phi difference are 0, and the full update reduces to
// phi' = phi, c' = c + D~ lap(c) with the same roundings. Warp-uniform.
template <int R2>
__device__ __forceinline__ bool band_is_bulk(const float (&bp)[R2], float& v) {
  v = __shfl_sync(0xffffffffu, bp[0], 0);
  bool b = (v == 1.f) | (v == 0.f);
#pragma unroll
  for (int j = 0; j < R2; ++j) b = b & (bp[j] == v);
  return __all_sync(0xffffffffu, b);
}

// The reduced update of a bulk band of R = 2 NP rows (rows y0 .. y0 + R - 1;
// bp / bcv hold rows y0 - 1 .. y0 + R).
template <int NP>
__device__ __forceinline__ void band_bulk_pk(const Coef<float>& k, const Geo& g,
                                             float* __restrict__ phi_out,
                                             float* __restrict__ c_out, int xs, int y0,
                                             const float (&bp)[2 * NP + 2],
                                             const float (&bcv)[2 * NP + 2], float v) {
  const int lane = threadIdx.x;
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + lane;
  const bool owner = lane >= 1 && lane <= kStrip && x < nx;
  const F2 Dv = sp(fmaf(k.a1, v, k.a0));
  float cw = shfl_w(bcv[1]), ce = shfl_e(bcv[1]);
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    const float cw2 = shfl_w(bcv[2 * j + 2]), ce2 = shfl_e(bcv[2 * j + 2]);
    const F2 cN = pk(bcv[2 * j], bcv[2 * j + 1]), c0 = pk(bcv[2 * j + 1], bcv[2 * j + 2]);
    const F2 cS = pk(bcv[2 * j + 2], bcv[2 * j + 3]);
    const F2 lc = fma2(sp(-2.f), c0, cN + cS) + fma2(sp(-2.f), c0, pk(cw, cw2) + pk(ce, ce2));
    const F2 c1 = c0 + Dv * lc;
    const int row = y0 + 2 * j;
    if (owner) {
      const int64_t o = (int64_t)row * g.pitch + x;
      if (row < ny) {
        phi_out[o] = bp[2 * j + 1];
        c_out[o] = lo(c1);
      }
      if (row + 1 < ny) {
        phi_out[o + g.pitch] = bp[2 * j + 2];
        c_out[o + g.pitch] = hi(c1);
      }
    }
    if (j + 1 < NP) {
      cw = shfl_w(bcv[2 * j + 3]);
      ce = shfl_e(bcv[2 * j + 3]);
    }
  }
}

// Noise words of a band from BandNoise (the blocks spread over the warp's
// lanes, words fetched by shuffles), drawn at the first row that needs any.
template <int ROWS>
struct ShuffleNoise {
  BandNoise<ROWS> b;
  uint64_t seed, step;
  int y0;
  uint32_t gbase;
  bool drawn;
  __device__ __forceinline__ ShuffleNoise(uint64_t seed_, uint64_t step_, int y0_,
                                          uint32_t gbase_)
      : seed(seed_), step(step_), y0(y0_), gbase(gbase_), drawn(false) {}
  // every lane of the warp calls this together
  __device__ __forceinline__ uint32_t word(int r, int x) {
    if (!drawn) {
      b.draw(seed, step, y0, gbase);
      drawn = true;
    }
    return b.word(r, x, gbase);
  }
};

// Noise words of a band from a table in shared memory that the CTA filled
// beforehand: words[(r * kGroups + i) * 4 + j] is word j of the Philox block
// (gbase + i, y0 + r, step).
struct TableNoise {
  const uint32_t* words;
  uint32_t gbase;
  __device__ __forceinline__ uint32_t word(int r, int x) const {
    int i = (int)((uint32_t)x / 4u - gbase);
    i = i < 0 ? 0 : (i >= kGroups ? kGroups - 1 : i);  // halo lanes: any valid entry
    return words[(r * kGroups + i) * 4 + (x & 3)];
  }
};

// Full update of a band of R = 2 NP rows, marched as NP row pairs: pair j
// holds output rows y0 + 2j (low half) and y0 + 2j + 1 (high half). bp / bcv
// hold phi / c of rows y0 - 1 .. y0 + R. The pointwise D~ and Q~ are
// evaluated once per loaded row pair and shared by the two output pairs that
// read them.
template <int NP, class Noise>
__device__ __forceinline__ void band_full_pk(const Coef<float>& k, const Geo& g,
                                             float* __restrict__ phi_out,
                                             float* __restrict__ c_out, Noise& noise, int xs,
                                             int y0, const float (&bp)[2 * NP + 2],
                                             const float (&bcv)[2 * NP + 2]) {
  const int lane = threadIdx.x;
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + lane;
  const bool owner = lane >= 1 && lane <= kStrip && x < nx;
  const F2 two = sp(2.f);
  const bool noisy = k.alpha != 0.f;

  // row pair (2j, 2j + 1) of bp: its point values and west / east phi
  F2 Dp, Qp;
  point2(k, pk(bp[0], bp[1]), pk(bcv[0], bcv[1]), Dp, Qp);
  float wa = shfl_w(bp[0]), ea = shfl_e(bp[0]), wb = shfl_w(bp[1]), eb = shfl_e(bp[1]);

#pragma unroll
  for (int j = 0; j < NP; ++j) {
    const float pa = bp[2 * j], pb = bp[2 * j + 1], pc = bp[2 * j + 2], pd = bp[2 * j + 3];
    const float ca = bcv[2 * j], cb = bcv[2 * j + 1], cc = bcv[2 * j + 2], cd = bcv[2 * j + 3];
    F2 Dn, Qn;
    point2(k, pk(pc, pd), pk(cc, cd), Dn, Qn);
    const float wc = shfl_w(pc), ec = shfl_e(pc), wd = shfl_w(pd), ed = shfl_e(pd);
    const F2 pN = pk(pa, pb), p0 = pk(pb, pc), pS = pk(pc, pd);
    const F2 cN = pk(ca, cb), c0 = pk(cb, cc), cS = pk(cc, cd);
    const F2 pNW = pk(wa, wb), pNE = pk(ea, eb);
    const F2 pW = pk(wb, wc), pE = pk(eb, ec);
    const F2 pSW = pk(wc, wd), pSE = pk(ec, ed);
    const F2 cW = pk(shfl_w(cb), shfl_w(cc)), cE = pk(shfl_e(cb), shfl_e(cc));
    const F2 DN = Dp, DS = Dn, QN = Qp, QS = Qn;
    const float D1 = hi(Dp), D2 = lo(Dn), Q1 = hi(Qp), Q2 = lo(Qn);
    const F2 D0 = pk(D1, D2), Q0 = pk(Q1, Q2);
    const F2 lc = fma2(sp(-2.f), c0, cN + cS) + fma2(sp(-2.f), c0, cW + cE);

    const F2 DW = pk(shfl_w(D1), shfl_w(D2)), DE = pk(shfl_e(D1), shfl_e(D2));
    const F2 QW = pk(shfl_w(Q1), shfl_w(Q2)), QE = pk(shfl_e(Q1), shfl_e(Q2));
    const F2 quarter = sp(0.25f);

    const F2 px = pN - pS;
    const F2 py = pW - pE;
    const F2 pxx = fma2(sp(-2.f), p0, pN + pS);
    const F2 pyy = fma2(sp(-2.f), p0, pW + pE);
    const F2 lp = pxx + pyy;
    const F2 pxy = quarter * ((pNW - pSW) - (pNE - pSE));

    // dc * dt (Warren1995.py:69-71); in bulk every added term is exactly 0
    const F2 fl = fma2(DW - DE, cW - cE, (DN - DS) * (cN - cS));
    F2 dc = fma2(quarter, fl, D0 * lc);
    dc = fma2(Q0, lp, dc);
    const F2 fq = fma2(QW - QE, py, (QN - QS) * px);
    dc = fma2(quarter, fq, dc);

    // anisotropy without trig: theta = atan2(py, px)
    const F2 r2 = fma2(px, px, py * py);
    const float r2a = lo(r2), r2b = hi(r2);
    const F2 n = pk(rsqrtf(fmaxf(r2a, 1e-30f)), rsqrtf(fmaxf(r2b, 1e-30f)));
    const F2 ux = px * n, uy = py * n;
    const F2 c2u = ux * ux - uy * uy;
    const F2 s2u = two * ux * uy;
    const bool ga = r2a > tiny_r2<float>(), gb = r2b > tiny_r2<float>();
    const F2 c2 = pk(ga ? lo(c2u) : 1.f, gb ? hi(c2u) : 1.f);
    const F2 s2 = pk(ga ? lo(s2u) : 0.f, gb ? hi(s2u) : 0.f);
    const F2 c4 = c2 * c2 - s2 * s2;
    const F2 s4 = two * s2 * c2;
    const F2 eta = fma2(sp(k.ye), c4, sp(1.f));
    const F2 etap = sp(-4.f * k.ye) * s4;
    const F2 etapp = sp(-16.f * k.ye) * c4;

    // dphi * dt (Warren1995.py:82-86)
    const F2 om = sp(1.f) - p0;
    const F2 g0 = p0 * p0 * (om * om);
    const F2 gp = p0 * fma2(p0, fma2(sp(4.f), p0, sp(-6.f)), two);
    const F2 HA = fma2(sp(k.WA), gp, sp(k.hA) * g0);
    const F2 HB = fma2(sp(k.WB), gp, sp(k.hB) * g0);
    const F2 oc = sp(1.f) - c0;
    const F2 Hs = fma2(oc, HA, c0 * HB);
    const F2 dtM = fma2(oc, sp(k.dtMA), c0 * sp(k.dtMB));
    const F2 dyx = pyy - pxx;
    const F2 t1 = eta * eta * lp;
    const F2 t2 = eta * etap * fma2(s2, dyx, two * c2 * pxy);
    const F2 t3 = sp(0.5f) * fma2(etap, etap, eta * etapp) *
                  fma2(c2, dyx, fma2(sp(-2.f), s2 * pxy, lp));
    const F2 aniso = t1 + t2 + t3;
    F2 dphi = dtM * (sp(k.e2) * aniso - Hs);

    // noise (:85-86) on cells with g(phi) != 0
    const float g0a = lo(g0), g0b = hi(g0);
    const bool need0 = noisy && owner && g0a != 0.f;
    const bool need1 = noisy && owner && g0b != 0.f;
    if (__any_sync(0xffffffffu, need0 || need1)) {
      const uint32_t wA = noise.word(2 * j, x), wB = noise.word(2 * j + 1, x);
      const F2 u = pk(float(wA >> 8) * 5.9604644775390625e-08f,
                      float(wB >> 8) * 5.9604644775390625e-08f);
      const F2 nz = dtM * sp(k.alpha) * fma2(two, u, sp(-1.f)) * (sp(16.f) * g0) * Hs;
      dphi = dphi + pk(need0 ? lo(nz) : 0.f, need1 ? hi(nz) : 0.f);
    }
    const F2 p1 = p0 + dphi;
    const F2 c1 = c0 + dc;
    const int row = y0 + 2 * j;
    if (owner) {
      const int64_t o = (int64_t)row * g.pitch + x;
      if (row < ny) {
        phi_out[o] = lo(p1);
        c_out[o] = lo(c1);
      }
      if (row + 1 < ny) {
        phi_out[o + g.pitch] = hi(p1);
        c_out[o + g.pitch] = hi(c1);
      }
    }
    Dp = Dn;
    Qp = Qn;
    wa = wc;
    ea = ec;
    wb = wd;
    eb = ed;
  }
}

// Band of R = 2 NP rows of the float kernel: the exact bulk form when the
// band is bulk, else the full update with noise words by shuffles.
template <int NP>
__device__ __forceinline__ void band_compute_pk(const Coef<float>& k, const Geo& g,
                                                float* __restrict__ phi_out,
                                                float* __restrict__ c_out, uint64_t seed,
                                                uint64_t step, int xs, int y0,
                                                const float (&bp)[2 * NP + 2],
                                                const float (&bcv)[2 * NP + 2]) {
  float v;
  if (k.bulk && band_is_bulk(bp, v)) {
    band_bulk_pk<NP>(k, g, phi_out, c_out, xs, y0, bp, bcv, v);
    return;
  }
  // first owned column's Philox block (owners are lanes 1..30, x >= 0)
  ShuffleNoise<2 * NP> noise(seed, step, y0, (uint32_t)(xs + 1) / 4u);
  band_full_pk<NP>(k, g, phi_out, c_out, noise, xs, y0, bp, bcv);
}

}  // namespace w95
}  // namespace ppf
