/* FP64 C restatement of the Warren1995 engine step, for grids the numpy
 * restatement is too slow for (1024 x 1024 for 1000 steps: minutes in numpy,
 * seconds here).
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle: GPU parity tests use it as
 * the checker. Nothing in the shipped package links or loads it.
 *
 * It follows oracle/restate.py::warren1995_step operation for operation,
 * which in turn follows engine_Warren1995 (Engines/Warren1995.py:50-92) and
 * its helpers _p, _g, _gprime (:17-28) and gradx/grady/gradxx/gradyy
 * (:30-48): every product and sum is evaluated in the order numpy evaluates
 * the reference's expressions (left to right, scalar factors first where
 * Python groups them), with atan2/cos/sin from the C library for the angle
 * terms. Build it with -ffp-contract=off (no fused multiply-add) so that
 * each operation rounds as numpy's does; tests/test_oracle.py pins it to the
 * numpy restatement. Ghost fill: Simulation.apply_boundary_conditions
 * (simulation.py:560-618) with every axis filled, axis 0 then axis 1.
 * Noise: Philox4x32-10 (Salmon et al., SC'11) keyed as oracle/philox.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double W_A, W_B, L_A, L_B, T, T_mA, T_mB, D_S, D_L, v_m, R, y_e, M_A, M_B, ebar, alpha;
  double ebar2; /* ebar ** 2 as Python computes it */
} WarrenParams;

enum { BC_PERIODIC = 0, BC_NEUMANN = 1, BC_DIRCHLET = 2 };

static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

/* Ghost fill of padded arrays (ny+2) x (nx+2); vals[f][axis][side]. */
static void fill_ghosts(double* const* f, int nf, int ny, int nx, const int* bc,
                        const double* vals, double dx) {
  const int W = nx + 2;
  for (int a = 0; a < 2; ++a)
    for (int j = 0; j < nf; ++j) {
      double* x = f[j];
      const double lo = vals ? vals[(j * 2 + a) * 2 + 0] : 0.0;
      const double hi = vals ? vals[(j * 2 + a) * 2 + 1] : 0.0;
      if (a == 0) {
        double* g0 = x;
        double* g1 = x + (size_t)(ny + 1) * W;
        const double* r1 = x + (size_t)1 * W;
        const double* r2 = x + (size_t)ny * W;
        for (int i = 0; i < W; ++i) {
          if (bc[0] == BC_PERIODIC) {
            g0[i] = r2[i];
            g1[i] = r1[i];
          } else if (bc[0] == BC_NEUMANN) {
            g0[i] = r1[i] - dx * lo;
            g1[i] = r2[i] + dx * hi;
          } else {
            g0[i] = lo;
            g1[i] = hi;
          }
        }
      } else {
        for (int r = 0; r < ny + 2; ++r) {
          double* row = x + (size_t)r * W;
          if (bc[1] == BC_PERIODIC) {
            row[0] = row[nx];
            row[nx + 1] = row[1];
          } else if (bc[1] == BC_NEUMANN) {
            row[0] = row[1] - dx * lo;
            row[nx + 1] = row[nx] + dx * hi;
          } else {
            row[0] = lo;
            row[nx + 1] = hi;
          }
        }
      }
    }
}

/* Advances padded phi, c ((ny+2) x (nx+2), ghosts filled) by `steps` steps
 * from absolute step index step0. Returns 0, or -1 if memory ran out. */
int ppf_oracle_warren_run(double* phi, double* c, int ny, int nx, const WarrenParams* p,
                          double dx, double dt, const int* bc, const double* vals,
                          uint64_t seed, uint64_t step0, int steps) {
  const int W = nx + 2;
  const size_t n = (size_t)(ny + 2) * W;
  double* DC = (double*)malloc(n * sizeof(double));
  double* tmp = (double*)malloc(n * sizeof(double));
  double* phx = (double*)malloc(n * sizeof(double));
  double* nphi = (double*)malloc(n * sizeof(double));
  double* nc = (double*)malloc(n * sizeof(double));
  if (!DC || !tmp || !phx || !nphi || !nc) {
    free(DC); free(tmp); free(phx); free(nphi); free(nc);
    return -1;
  }
  /* scalar factors as Python groups them in the reference's expressions */
  const double hA = 30 * p->L_A * (1 / p->T - 1 / p->T_mA);
  const double hB = 30 * p->L_B * (1 / p->T - 1 / p->T_mB);
  const double two_dx = 2 * dx;
  const double dx2 = dx * dx;
  const double dLS = p->D_L - p->D_S;
  const double ebar2 = p->ebar2;
  const double m4ye = -4 * p->y_e;
  const double half_e2 = 0.5 * ebar2;
  double* fl[2] = {phi, c};

  for (int s = 0; s < steps; ++s) {
    const uint64_t step = step0 + (uint64_t)s;
    /* pointwise D_C, temp and phix over the whole padded array */
#pragma omp parallel for schedule(static)
    for (int r = 0; r < ny + 2; ++r) {
      for (int q = 0; q < W; ++q) {
        const size_t o = (size_t)r * W + q;
        const double f = phi[o], cc = c[o];
        const double g = f * f * (1 - f) * (1 - f);
        const double pp = f * f * f * (10 - 15 * f + 6 * f * f);
        const double gp = 4 * f * f * f - 6 * f * f + 2 * f;
        const double HA = p->W_A * gp + hA * g;
        const double HB = p->W_B * gp + hB * g;
        const double dcv = p->D_S + pp * dLS;
        DC[o] = dcv;
        tmp[o] = dcv * p->v_m * cc * (1 - cc) * (HB - HA) / p->R;
        if (r >= 1 && r <= ny)
          phx[o] = (phi[o - W] - phi[o + W]) / two_dx;
        else
          phx[o] = 0.0;
      }
    }
#pragma omp parallel for schedule(static)
    for (int r = 1; r <= ny; ++r) {
      for (int q = 1; q <= nx; ++q) {
        const size_t o = (size_t)r * W + q;
        const double f = phi[o], cc = c[o];
        const double g = f * f * (1 - f) * (1 - f);
        const double gp = 4 * f * f * f - 6 * f * f + 2 * f;
        const double HA = p->W_A * gp + hA * g;
        const double HB = p->W_B * gp + hB * g;
        const double fN = phi[o - W], fS = phi[o + W], fW = phi[o - 1], fE = phi[o + 1];
        const double phixx = (fN + fS - 2 * f) / dx2;
        const double phiyy = (fW + fE - 2 * f) / dx2;
        const double lphi = phixx + phiyy;
        const double phix = (fN - fS) / two_dx;
        const double phiy = (fW - fE) / two_dx;
        const double phixy = (phx[o - 1] - phx[o + 1]) / two_dx;
        const double cN = c[o - W], cS = c[o + W], cW = c[o - 1], cE = c[o + 1];
        const double cxx = (cN + cS - 2 * cc) / dx2;
        const double cyy = (cW + cE - 2 * cc) / dx2;
        const double dCx = (DC[o - W] - DC[o + W]) / two_dx;
        const double dCy = (DC[o - 1] - DC[o + 1]) / two_dx;
        const double cx = (cN - cS) / two_dx;
        const double cy = (cW - cE) / two_dx;
        const double tx = (tmp[o - W] - tmp[o + W]) / two_dx;
        const double ty = (tmp[o - 1] - tmp[o + 1]) / two_dx;
        const double deltac = DC[o] * (cxx + cyy) + (dCx * cx + dCy * cy) + tmp[o] * lphi +
                              (tx * phix + ty * phiy);
        const double theta = atan2(phiy, phix);
        const double eta = 1 + p->y_e * cos(4 * theta);
        const double etap = m4ye * sin(4 * theta);
        const double etapp = -16 * (eta - 1);
        const double c2 = cos(2 * theta);
        const double s2 = sin(2 * theta);
        const double Mphi = (1 - cc) * p->M_A + cc * p->M_B;
        double dphi = Mphi * ((ebar2 * eta * eta * lphi - (1 - cc) * HA - cc * HB) +
                              ebar2 * eta * etap * (s2 * (phiyy - phixx) + 2 * c2 * phixy) +
                              half_e2 * (etap * etap + eta * etapp) *
                                  (-2 * s2 * phixy + lphi + c2 * (phiyy - phixx)));
        if (p->alpha != 0) {
          const int col = q - 1, row = r - 1;
          uint32_t ctr[4] = {(uint32_t)(col / 4), (uint32_t)row, (uint32_t)step,
                             (uint32_t)(step >> 32)};
          philox(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
          const double u = (double)(ctr[col % 4] >> 8) * 5.9604644775390625e-08;
          const double rnd = 2 * u - 1;
          dphi += Mphi * p->alpha * rnd * (16 * g) * ((1 - cc) * HA + cc * HB);
        }
        nphi[o] = f + dphi * dt;
        nc[o] = cc + deltac * dt;
      }
    }
#pragma omp parallel for schedule(static)
    for (int r = 1; r <= ny; ++r) {
      memcpy(phi + (size_t)r * W + 1, nphi + (size_t)r * W + 1, (size_t)nx * sizeof(double));
      memcpy(c + (size_t)r * W + 1, nc + (size_t)r * W + 1, (size_t)nx * sizeof(double));
    }
    fill_ghosts(fl, 2, ny, nx, bc, vals, dx);
  }
  free(DC); free(tmp); free(phx); free(nphi); free(nc);
  return 0;
}

/* Ghost fill alone (tests). */
int ppf_oracle_fill_ghosts(double* phi, double* c, int ny, int nx, const int* bc,
                           const double* vals, double dx) {
  double* fl[2] = {phi, c};
  fill_ghosts(fl, 2, ny, nx, bc, vals, dx);
  return 0;
}
