/*
 * ppf_gb300.h -- C ABI of libppf_gb300.so, the GB300 (sm_103a) explicit
 * time-stepping engine behind pyphasefield's Simulation/engine plugin API.
 *
 * Conventions
 *  - Every function returns int32_t: PPF_OK (0) or a negative PPF_ERR_* code;
 *    ppf_last_error() gives a one-line message for the calling thread.
 *  - The library owns no field buffers. Callers pass device pointers, the
 *    grid geometry and a cudaStream_t (passed as void*, NULL = legacy default
 *    stream). Work is stream-ordered; no function synchronises the device.
 *  - Grids are C order, interior cells only (no ghost layers): axis ndim-1 is
 *    contiguous, rows are `pitch` elements apart, planes pitch*shape[ndim-2]
 *    elements apart. A 1-D grid is passed as 2-D with shape[0] = 1 and a
 *    periodic axis 0. Ghost cells of the reference's Field (pyphasefield
 *    field.py:6-20) are never stored: the boundary rule of
 *    Simulation.apply_boundary_conditions (simulation.py:560-618) is applied
 *    while each tile is loaded.
 *  - Input and output buffers of a step must not overlap.
 *  - *_f32 entry points store and compute in float, *_f64 in double. The
 *    physical parameters are always passed as double and folded on the host.
 */
#ifndef PPF_GB300_H
#define PPF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPF_ABI_VERSION 3

#define PPF_OK 0
#define PPF_ERR_INVALID (-1)     /* bad argument (shape, pitch, pointer, depth) */
#define PPF_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define PPF_ERR_UNSUPPORTED (-3) /* valid request the library does not implement */
#define PPF_ERR_TIMEOUT (-4)     /* a bounded device-side wait gave up */
#define PPF_ERR_NONFINITE (-5)   /* a field produced NaN/Inf (status flag) */

/* Boundary condition types, per axis. Spelled as in the reference
 * (Simulation.init_boundary_conditions, simulation.py:109-123). */
#define PPF_BC_PERIODIC 0
#define PPF_BC_NEUMANN 1
#define PPF_BC_DIRCHLET 2

/* Status-flag bits written by kernels into a caller-provided int32. */
#define PPF_STATUS_NONFINITE 1
#define PPF_STATUS_TIMEOUT 2
#define PPF_STATUS_RANGE 4
#define PPF_STATUS_NOT_CONVERGED 8 /* an iterative solve hit its iteration cap */

typedef struct PpfGrid {
  int32_t ndim;     /* 2 or 3 */
  int32_t reserved; /* must be 0 */
  int64_t shape[3]; /* interior cells per axis, C order (first ndim used) */
  int64_t pitch;    /* elements between rows; >= shape[ndim-1], multiple of 4 */
} PpfGrid;

/* Ghost-cell rule per axis (C order, same as PpfGrid.shape). value holds,
 * per field (up to 2), axis and side (0 = low, 1 = high), the Neumann
 * gradient (ghost = edge -/+ dx*value, simulation.py:583-584) or the
 * Dirichlet ghost value (simulation.py:591-592). The reference keeps these
 * in Simulation._boundary_conditions_array; this ABI takes one constant per
 * face. Corner ghosts compose axis by axis in the reference's fill order. */
typedef struct PpfBoundary {
  int32_t type[3];
  int32_t reserved;
  double value[2][3][2];
} PpfBoundary;

/* Diffusion explicit step: c += dt*D*lap(c)
 * (engine_ExplicitDiffusion, Engines/Diffusion.py:198-208). */
typedef struct PpfDiffusionParams {
  double dx, dt, D;
} PpfDiffusionParams;

/* Allen-Cahn ("CahnAllen") explicit step:
 * phi += dt*M*(eps^2 lap(phi) - 16 W (4phi^3 - 6phi^2 + 2phi))
 * (engine_CahnAllenExplicit, Engines/CahnAllen.py:128-135). */
typedef struct PpfAllenCahnParams {
  double dx, dt, M, epsilon, W;
} PpfAllenCahnParams;

/* Cahn-Hilliard explicit step:
 * mu = -eps^2 lap(c) + (4c^3 - 6c^2 + 2c);  c += dt*M*lap(mu)
 * (engine_CahnHilliardExplicit, Engines/CahnHilliard.py:134-146; the
 * reference omits dt, this ABI applies it), written in flux form: every
 * face flux dt*M*(mu_nbr - mu)/dx^2 is added to one cell and subtracted
 * from the other.
 * centered = 1: the buffers hold u = c - 1/2 (the double well's midpoint)
 *   and mu's bulk term is evaluated as 4u^3 - u (the same polynomial).
 * quantum > 0 (a power of two, float path only): every face flux is rounded
 *   to a multiple of quantum. With field values that are multiples of
 *   quantum below 2^24*quantum in magnitude, every float add is exact and
 *   the field's sum is conserved exactly (centered storage with
 *   quantum = 2^-24 covers c in (-1/2, 3/2)). 0 disables rounding. */
typedef struct PpfCahnHilliardParams {
  double dx, dt, M, epsilon, quantum;
  int32_t centered;
  int32_t reserved;
} PpfCahnHilliardParams;

/* Warren-Boettinger 1995 Ni-Cu isothermal solidification
 * (engine_Warren1995, Engines/Warren1995.py:50-92). Material constants are
 * the Warren1995 engine's user_data keys (Warren1995.py:138-169); ebar, W_A,
 * W_B, M_A, M_B are the derived values of just_before_simulating
 * (Warren1995.py:193-203). The noise draw U[0,1) of cell (row, col) at a
 * step is word col % 4 of Philox4x32-10 with counter (col / 4, row, step)
 * and key seed, top 24 bits times 2^-24 (replacing np.random.random, :85). */
typedef struct PpfWarren1995Params {
  double dx, dt;
  double T_mA, T_mB, L_A, L_B, D_L, D_S, v_m, R, y_e, T, alpha;
  double ebar, W_A, W_B, M_A, M_B;
} PpfWarren1995Params;

/* Launch shape of one explicit-step call. NULL selects the defaults
 * (depth 1, library-chosen tile). depth = time steps advanced per HBM pass
 * (temporal blocking, 1..8, 2-D Diffusion/Allen-Cahn only); tile_x/tile_y =
 * output tile per CTA (0 = default; for Warren1995 tile_y is the number of
 * rows each warp walks: 2, 4, 8 or 16); pdl = 1 launches with programmatic
 * dependent launch so back-to-back steps overlap their launch latency;
 * flags = PPF_TILING_* bits; zchunk (3-D kernels) = planes per CTA along z,
 * 0 = chosen by the library. */
typedef struct PpfTiling {
  int32_t depth;
  int32_t tile_x;
  int32_t tile_y;
  int32_t pdl;
  int32_t flags;
  int32_t zchunk;
} PpfTiling;

/* Warren1995: evaluate the full update on every cell. Without this flag a
 * row of cells whose 3x3 neighbourhoods are all exactly phi = 1 (or all
 * exactly 0) takes the exact reduced form phi' = phi, c' = c + D~ lap(c),
 * bit-identical to the full form there (every phi term is exactly zero). */
#define PPF_TILING_FULL_EVAL 1

/* ---- library ---------------------------------------------------------- */

/* ABI version (PPF_ABI_VERSION) and build string. */
int32_t ppf_version(int32_t* abi_version, char* buf, size_t len);
/* Message of the last failed call on this thread (empty if none). */
int32_t ppf_last_error(char* buf, size_t len);
/* Device properties the host side uses for tiling: SM count, max shared
 * memory per block (opt-in) and compute capability. */
int32_t ppf_device_info(int32_t device, int32_t* sm_count, int32_t* smem_optin,
                        int32_t* cc_major, int32_t* cc_minor);

/* ---- explicit steps (one HBM pass) ------------------------------------ */

/* Advance tiling->depth time steps in one pass. Replaces Simulation.simulation_loop() +
 * apply_boundary_conditions() of the Diffusion engine
 * (simulation.py:262-266, Engines/Diffusion.py:198-208). */
int32_t ppf_diffusion_step_f32(const PpfDiffusionParams* p, const PpfGrid* g,
                               const PpfBoundary* bc, const float* in,
                               float* out, const PpfTiling* tiling,
                               void* stream);
int32_t ppf_diffusion_step_f64(const PpfDiffusionParams* p, const PpfGrid* g,
                               const PpfBoundary* bc, const double* in,
                               double* out, const PpfTiling* tiling,
                               void* stream);

/* Same contract for the Allen-Cahn engine (Engines/CahnAllen.py:128-135). */
int32_t ppf_allen_cahn_step_f32(const PpfAllenCahnParams* p, const PpfGrid* g,
                                const PpfBoundary* bc, const float* in,
                                float* out, const PpfTiling* tiling,
                               void* stream);
int32_t ppf_allen_cahn_step_f64(const PpfAllenCahnParams* p, const PpfGrid* g,
                                const PpfBoundary* bc, const double* in,
                                double* out, const PpfTiling* tiling,
                               void* stream);

/* One Cahn-Hilliard step (Engines/CahnHilliard.py:134-146), radius-2
 * stencil through an on-chip mu tile. mass_accum (nullable) receives
 * += sum of the new field in double. status (nullable) gets
 * PPF_STATUS_NONFINITE / PPF_STATUS_RANGE bits or'ed in. */
int32_t ppf_cahn_hilliard_step_f32(const PpfCahnHilliardParams* p,
                                   const PpfGrid* g, const PpfBoundary* bc,
                                   const float* in, float* out,
                                   double* mass_accum, int32_t* status,
                                   const PpfTiling* tiling, void* stream);
int32_t ppf_cahn_hilliard_step_f64(const PpfCahnHilliardParams* p,
                                   const PpfGrid* g, const PpfBoundary* bc,
                                   const double* in, double* out,
                                   double* mass_accum, int32_t* status,
                                   const PpfTiling* tiling, void* stream);

/* One Warren1995 step of (phi, c) (Engines/Warren1995.py:50-92), 2-D only.
 * The noise of a step is keyed by step + (*step_base if step_base is not
 * NULL): a captured graph of several steps passes fixed offsets and a device
 * counter advanced by ppf_counter_add_u64 after each replay. */
int32_t ppf_warren1995_step_f32(const PpfWarren1995Params* p, const PpfGrid* g,
                                const PpfBoundary* bc, const float* phi_in,
                                const float* c_in, float* phi_out, float* c_out,
                                uint64_t seed, uint64_t step,
                                const uint64_t* step_base,
                                const PpfTiling* tiling, void* stream);
int32_t ppf_warren1995_step_f64(const PpfWarren1995Params* p, const PpfGrid* g,
                                const PpfBoundary* bc, const double* phi_in,
                                const double* c_in, double* phi_out,
                                double* c_out, uint64_t seed, uint64_t step,
                                const uint64_t* step_base,
                                const PpfTiling* tiling, void* stream);

/* ---- implicit and Crank-Nicolson diffusion ------------------------------ */

/* Solver choice of the Diffusion engine's user_data["solver"]
 * (Diffusion.simulation_loop, Engines/Diffusion.py:671-720). */
#define PPF_SOLVER_EXPLICIT 0
#define PPF_SOLVER_IMPLICIT 1
#define PPF_SOLVER_CRANK_NICOLSON 2
#define PPF_SOLVER_IMEX 3

/* One step of engine_ImplicitDiffusion{1,2,3}D[_ADI][_GMRES] or
 * engine_CrankNicolsonDiffusion{1,2,3}D[_ADI][_GMRES]
 * (Engines/Diffusion.py:210-633). Every axis is periodic, whatever the
 * simulation's boundary conditions: the reference's matrices are
 * (diffusion_matrix_1d/_2d/_3d, :18-196). a = D dt / dx^2 (implicit) or
 * D dt / (2 dx^2) (Crank-Nicolson).
 * adi = 1: 1-D solves axis by axis in the reference's order; exact up to
 *   rounding. adi = 0 (2-D / 3-D): the full (1 + 2 d a) I - a sum(S + S^-1)
 *   system by Chebyshev semi-iteration with the iteration count that bounds
 *   the error by tol relative to the field (tol = 0: 1e-7 float, 1e-14
 *   double). The *_GMRES engines solve the same systems approximately
 *   (scipy gmres, residual 1e-5 relative); they map to the same call.
 * A 2-D grid with shape[0] = 1 is the 1-D engine. */
typedef struct PpfImplicitDiffusionParams {
  double dx, dt, D;
  double tol;
  int32_t solver; /* PPF_SOLVER_IMPLICIT or PPF_SOLVER_CRANK_NICOLSON */
  int32_t adi;
} PpfImplicitDiffusionParams;

/* Bytes of device scratch a line solve along any axis of g needs. */
int32_t ppf_implicit_scratch_bytes(const PpfGrid* g, int32_t elem_bytes, size_t* bytes);
/* in and out must differ. tmp: a third field of g's geometry, needed by
 * Crank-Nicolson with adi = 1 and by every adi = 0 solve in 2-D / 3-D
 * (may be NULL otherwise). iterations (nullable) receives the Chebyshev
 * iteration count (0 for line solves). */
int32_t ppf_diffusion_implicit_step_f32(const PpfImplicitDiffusionParams* p,
                                        const PpfGrid* g, const float* in,
                                        float* out, float* tmp, void* scratch,
                                        size_t scratch_bytes, int32_t* iterations,
                                        void* stream);
int32_t ppf_diffusion_implicit_step_f64(const PpfImplicitDiffusionParams* p,
                                        const PpfGrid* g, const double* in,
                                        double* out, double* tmp, void* scratch,
                                        size_t scratch_bytes, int32_t* iterations,
                                        void* stream);
/* The building blocks. Line solve along `axis` (C order) of every line:
 * (1 + 2 alpha) x_i - alpha (x_{i-1} + x_{i+1}) = d_i, periodic, with
 * d = in (expl_axis < 0) or d = (1 - 2 expl_alpha) in + expl_alpha
 * (in[-1] + in[+1]) along expl_axis (the explicit half steps of the
 * Crank-Nicolson ADI engines, Diffusion.py:527, 580-590). In place
 * (in == out) only without an explicit part. >= 3 cells along the axis. */
int32_t ppf_line_solve_f32(const PpfGrid* g, int32_t axis, double alpha,
                           int32_t expl_axis, double expl_alpha, const float* in,
                           float* out, void* scratch, size_t scratch_bytes,
                           void* stream);
int32_t ppf_line_solve_f64(const PpfGrid* g, int32_t axis, double alpha,
                           int32_t expl_axis, double expl_alpha, const double* in,
                           double* out, void* scratch, size_t scratch_bytes,
                           void* stream);
/* Full periodic solve (1 + 2 d alpha) x - alpha sum(neighbours of x) = b,
 * b = in (rhs_alpha = 0) or (1 - 2 d rhs_alpha) in + rhs_alpha
 * sum(neighbours of in); in, out, tmp distinct. */
int32_t ppf_periodic_solve_f32(const PpfGrid* g, double alpha, double rhs_alpha,
                               double tol, const float* in, float* out, float* tmp,
                               int32_t* iterations, void* stream);
int32_t ppf_periodic_solve_f64(const PpfGrid* g, double alpha, double rhs_alpha,
                               double tol, const double* in, double* out,
                               double* tmp, int32_t* iterations, void* stream);

/* One step of the Allen-Cahn ("CahnAllen") or Cahn-Hilliard engines with
 * user_data solver "implicit", "crank-nicolson" or "imex"
 * (Engines/CahnAllen.py:137-267, dispatch :325-361;
 * Engines/CahnHilliard.py:148-341, dispatch :382-421). Periodic on every
 * axis, as the reference's matrices are. a = M dt eps^2 / dx^2.
 *  Allen-Cahn, 1-D implicit: (1 + 2a + 16 W M dt g(phi)) on the diagonal,
 *    g(phi) = 4 phi^2 - 6 phi + 2; 2-D implicit: rows then columns with
 *    8 W M dt g (ADI; gmres without adi: the full 2-D system by Chebyshev
 *    with Jacobi scaling, error bound tol, needs 4 W M dt < 1); 3-D implicit:
 *    x, y, z solves whose diagonal is the first n entries of the flattened
 *    source term, as np.fill_diagonal gives the reference; Crank-Nicolson
 *    (2-D): explicit half and solve along x, then along y; IMEX (1-D).
 *    Branches the reference leaves empty return the field unchanged.
 *  Cahn-Hilliard, 1-D implicit and Crank-Nicolson: the cyclic pentadiagonal
 *    system of CahnHilliard.py:20-71. Its 2-D / 3-D and IMEX engines call
 *    an Allen-Cahn matrix builder the module lacks (TypeError in the
 *    reference); they run the Allen-Cahn formulas they copy.
 * tmp: a third field (Crank-Nicolson, IMEX, the full 2-D solve). */
#define PPF_MODEL_CAHN_HILLIARD 3
typedef struct PpfImplicitPhaseParams {
  double dx, dt, M, W, epsilon;
  double tol;
  int32_t model;  /* PPF_MODEL_ALLEN_CAHN or PPF_MODEL_CAHN_HILLIARD */
  int32_t solver; /* PPF_SOLVER_IMPLICIT, _CRANK_NICOLSON or _IMEX */
  int32_t adi, gmres;
  int32_t max_iter; /* MINRES iteration cap (0: 20000); past it the solve
                       sets PPF_STATUS_NOT_CONVERGED */
  int32_t reserved;
} PpfImplicitPhaseParams;

int32_t ppf_phase_implicit_scratch_bytes(const PpfGrid* g, int32_t elem_bytes, size_t* bytes);
int32_t ppf_phase_implicit_step_f32(const PpfImplicitPhaseParams* p, const PpfGrid* g,
                                    const float* in, float* out, float* tmp, void* scratch,
                                    size_t scratch_bytes, int32_t* iterations, void* stream);
int32_t ppf_phase_implicit_step_f64(const PpfImplicitPhaseParams* p, const PpfGrid* g,
                                    const double* in, double* out, double* tmp, void* scratch,
                                    size_t scratch_bytes, int32_t* iterations, void* stream);
/* Periodic line solve along `axis` with a diagonal that varies:
 * d_i x_i - alpha (x_{i-1} + x_{i+1}) = b_i, d_i = dvec[i] (dvec non-NULL:
 * one diagonal for every line, indexed by the position along it) or
 * dbase + dcoef (4 b_i^2 - 6 b_i + 2); b = in, or with expl = 1 the
 * explicit half step (1 - 2 expl_alpha) in + expl_alpha (in[-1] + in[+1])
 * along the same axis. In place (in == out) only without expl. */
int32_t ppf_var_line_solve_f32(const PpfGrid* g, int32_t axis, double alpha, double dbase,
                               double dcoef, const float* dvec, int32_t expl,
                               double expl_alpha, const float* in, float* out, void* scratch,
                               size_t scratch_bytes, void* stream);
int32_t ppf_var_line_solve_f64(const PpfGrid* g, int32_t axis, double alpha, double dbase,
                               double dcoef, const double* dvec, int32_t expl,
                               double expl_alpha, const double* in, double* out, void* scratch,
                               size_t scratch_bytes, void* stream);

/* ---- NCGPU (multi-component solidification with orientation) ----------- */

/* One step of the NCGPU engine (Engines/NCGPU.py:37-303, simulation_loop
 * :499-532), 2 to PPF_NCGPU_MAX_COMP components (ncomp), 2-D: fields phi, q1, q4 and the
 * fractions c_1 .. c_{ncomp-1} of all but the last component (the last is
 * 1 - sum c), 3 + ncomp - 1 pointers in fields_in / fields_out. Parameters as
 * NCGPU.init_tdb_params derives them (:336-373): ebar2 = 6 sqrt(2) S[1] d /
 * T_M[1], W and M per component (components sorted). gibbs[phase][comp]
 * holds up to 4 temperature ranges of the pure element's Gibbs energy in
 * J/mol, {T_lo, T_hi, c_1, c_T, c_TlnT, c_T^2, c_T^3, c_T^7, c_1/T, c_T^-9}
 * (phase 0 = the solid, the first phase name in sorted order; 1 = liquid);
 * the molar Gibbs energy adds R T sum_i x_i ln x_i, R = 8.3145, and the
 * binary Redlich-Kister terms of `excess`.
 * noise_scale multiplies the Langevin term of dF/dc (1 = the reference);
 * its N(0,1) numbers come from Philox4x32-10 keyed by (seed, step
 * (+ *step_base), cell). temperature: a field of the grid's layout.
 * transfer: device scratch of 2 ncomp - 1 fields of the grid's layout.
 * Boundaries: periodic or zero-gradient Neumann. As the reference, dG/dc is
 * one forward difference per cell (the first component up, the last down)
 * shared by every component. */
#define PPF_NCGPU_MAX_COMP 6
/* Engines/NCGPU.py, and Engines/NCGPU_new.py (per-component dG/dc and
 * concentration noise, phase noise sqrt(2 R T M_phi / v_m) noise_phi added
 * after the mobility, orientation noise sqrt(1e-10 R T / v_m) noise_q in the
 * quaternion brackets, phi clamped to [1e-4, 0.9999]) */
#define PPF_NCGPU_VARIANT_NCGPU 0
#define PPF_NCGPU_VARIANT_NEW 1
#define PPF_NCGPU_MAX_EXCESS 16
/* One binary Redlich-Kister term of a phase: x_a x_b L(T) (x_a - x_b)^order
 * added to its molar Gibbs energy, L piecewise in T as the gibbs ranges. */
typedef struct PpfNcgpuExcess {
  int32_t phase;      /* 0 the solid, 1 the liquid */
  int32_t a, b;       /* component indices (sorted order), a != b */
  int32_t order;      /* k >= 0 */
  int32_t npieces;    /* temperature ranges in piece, 0..4 */
  int32_t reserved;
  double piece[4][10];
} PpfNcgpuExcess;
typedef struct PpfNcgpuParams {
  double dx, dt, v_m, D_L, D_S, M_qmax, H, y_e, beta, ebar2, noise_scale;
  double W[PPF_NCGPU_MAX_COMP], M[PPF_NCGPU_MAX_COMP];
  double gibbs[2][PPF_NCGPU_MAX_COMP][4][10];
  int32_t npieces[2][PPF_NCGPU_MAX_COMP];
  int32_t ncomp;
  int32_t nexcess;    /* 0..PPF_NCGPU_MAX_EXCESS terms in excess */
  PpfNcgpuExcess excess[PPF_NCGPU_MAX_EXCESS];
  int32_t variant;    /* PPF_NCGPU_VARIANT_NCGPU or PPF_NCGPU_VARIANT_NEW */
  int32_t reserved;
  /* PPF_NCGPU_VARIANT_NEW only: eqbar^2 (the orientation gradient energy;
   * NCGPU uses ebar2 / 4) and the phase and orientation noise amplitudes
   * (noise_scale is the concentration noise's) */
  double eqbar2, noise_phi, noise_q;
} PpfNcgpuParams;

int32_t ppf_ncgpu_step_f32(const PpfNcgpuParams* p, const PpfGrid* g, const PpfBoundary* bc,
                           const float* const* fields_in, float* const* fields_out,
                           const float* temperature, const double* tables, float* transfer,
                           uint64_t seed, uint64_t step, const uint64_t* step_base, void* stream);
int32_t ppf_ncgpu_step_f64(const PpfNcgpuParams* p, const PpfGrid* g, const PpfBoundary* bc,
                           const double* const* fields_in, double* const* fields_out,
                           const double* temperature, const double* tables, double* transfer,
                           uint64_t seed, uint64_t step, const uint64_t* step_base, void* stream);

/* The pure-element Gibbs energies of both phases and the interaction
 * parameters at every cell's temperature, for a temperature field that
 * stays fixed over many steps. The caller allocates 2 ncomp + nexcess
 * planes of doubles in the grid's layout (rows x pitch each). _f64 fills
 * them: plane l = G(solid, component l), plane ncomp + l = G(liquid, l),
 * plane 2 ncomp + e = L of excess[e]. _f32 fills the same memory with
 * 3 ncomp - 2 + nexcess planes of floats (each rows x pitch floats):
 * G(solid, l) - G(liquid, l) for l < ncomp, then G(solid, l) - G(solid,
 * last) and G(liquid, l) - G(liquid, last) for l < ncomp - 1, then L of
 * excess[e] (the differences formed in double). Passed as `tables` to
 * ppf_ncgpu_step_* of the same precision, the step reads them instead of
 * evaluating the piecewise polynomials (NULL: evaluated every step, the
 * same values). Recompute them whenever the temperature changes. */
int32_t ppf_ncgpu_tables_f32(const PpfNcgpuParams* p, const PpfGrid* g, const float* temperature,
                             double* tables, void* stream);
int32_t ppf_ncgpu_tables_f64(const PpfNcgpuParams* p, const PpfGrid* g, const double* temperature,
                             double* tables, void* stream);
/* temperature += dT on every interior cell (stream-ordered): the
 * per-step rise of a LINEAR_GRADIENT temperature with dT/dt, dT = dTdt * dt
 * (update_thermal_gradient_2D_kernel, ppf_gpu_utils.py:326-334, which
 * Simulation.simulate runs after every engine step, simulation.py:262-266).
 * Tables from ppf_ncgpu_tables_* do not follow it: step without them. */
int32_t ppf_ncgpu_temperature_advance_f32(const PpfGrid* g, float* temperature, double dT,
                                          void* stream);
int32_t ppf_ncgpu_temperature_advance_f64(const PpfGrid* g, double* temperature, double dT,
                                          void* stream);

/* ---- batched ensemble ------------------------------------------------- */

#define PPF_MODEL_WARREN1995 1
#define PPF_MODEL_ALLEN_CAHN 2

/* One ensemble member: an independent 2-D float grid with its own ping-pong
 * buffers and parameters (one reference Simulation instance each). Step
 * parity p reads phi[p] (and c[p]) and writes phi[1-p] (and c[1-p]). */
typedef struct PpfMember {
  int32_t model; /* PPF_MODEL_* */
  int32_t reserved;
  int64_t ny, nx, pitch;
  PpfBoundary bc;
  float* phi[2];
  float* c[2]; /* Warren1995 only */
  uint64_t seed;
  PpfWarren1995Params w95; /* Warren1995 only */
  PpfAllenCahnParams ac;   /* Allen-Cahn only */
} PpfMember;

typedef struct PpfEnsemblePlan {
  const void* device_table; /* caller device memory holding the member table */
  int64_t n_items;          /* warp bands over all members */
  int32_t n_members;
  int32_t rows;    /* rows per warp band (tiling->tile_y: 2, 4 or 8) */
  int64_t n_units; /* units of 4 x bands bands (one CTA pass each) */
  int32_t bands;   /* bands per warp and unit (tiling->tile_x: 1 or 4, with two
                      rows also 8 or 16; 0 -> 4) */
  int32_t reserved;
} PpfEnsemblePlan;

/* Device bytes of the member table (members and unit map) for these
 * members. */
int32_t ppf_ensemble_plan_bytes(const PpfMember* members, int32_t n,
                                const PpfTiling* tiling, size_t* bytes);
/* Validates the members, folds their parameters and copies the table into
 * device_table (waits for that copy on `stream`). */
int32_t ppf_ensemble_build(const PpfMember* members, int32_t n,
                           const PpfTiling* tiling, void* device_table,
                           size_t bytes, PpfEnsemblePlan* plan, void* stream);
/* One time step of every member in one launch; Warren1995 noise keyed by
 * (member seed, step + *step_base). Replaces the per-instance
 * Simulation.simulate loop (simulation.py:245-271) over the reference's
 * engine_Warren1995 / engine_CahnAllenExplicit. */
int32_t ppf_ensemble_step_f32(const PpfEnsemblePlan* plan, int32_t parity,
                              uint64_t step, const uint64_t* step_base,
                              const PpfTiling* tiling, void* stream);
/* nsteps time steps of every member. Two-row plans, and four- and
 * eight-row plans given no `sync` (NULL): one launch per step (programmatic
 * dependent launch when tiling->pdl). Four- and eight-row plans given a
 * `sync` buffer: ONE persistent cooperative launch: the CTAs meet at a grid
 * barrier between steps (waits bounded; a timeout sets PPF_STATUS_TIMEOUT in
 * the status word and ends the launch early). `sync` is then caller device
 * memory of 8 bytes (8-byte aligned), zeroed once before its first use and
 * used by one launch at a time; after a timeout zero it again. Both ways give
 * the same results bit for bit. The member buffers swap by step parity,
 * starting from `parity`. */
int32_t ppf_ensemble_run_f32(const PpfEnsemblePlan* plan, int32_t parity,
                             uint64_t step, const uint64_t* step_base,
                             int32_t nsteps, void* sync, const PpfTiling* tiling,
                             void* stream);

/* ---- learned surrogate (no counterpart in the reference) --------------- *
 * A convolutional encoder-decoder that advances a Warren1995 (phi, c) state
 * by k stencil steps: patchify conv (P x P, stride P) -> L blocks of
 * [depthwise 3x3 conv, 1x1 conv C->E, GELU, 1x1 conv E->C, residual] ->
 * unpatchify conv predicting the normalised k-step change. The patch and 1x1
 * convolutions are implicit GEMMs on BF16 tensor cores (mma.sync m16n8k16,
 * FP32 accumulation); the patch gather / scatter happens in the GEMM's
 * operand loader and epilogue. Activations are channels-last [token][ch];
 * fields are [b][ch][H][pitch] float. Weights W[out][in] (bf16 for the
 * GEMMs). Gradient entry points accumulate (+=) into fp32 buffers. */
typedef struct PpfSgShape {
  int32_t B, H, W, pitch, P, C, E;
  float s0, s1;                          /* change scale of phi and c */
  float in_off0, in_sc0, in_off1, in_sc1; /* input (v - off) * sc */
  float lo0, hi0, lo1, hi1;               /* predictions clamped to [lo, hi] */
} PpfSgShape;

int32_t ppf_sg_gemm(const void* a, long long sam, long long sak, const void* b,
                    long long sbk, long long sbn, float* y, long long ldy,
                    const float* bias, int32_t accumulate, long long M,
                    long long N, long long K, int32_t splits, void* stream);
int32_t ppf_sg_patch_fwd(const PpfSgShape* s, const float* fields,
                         const void* w_in_bf16, const float* b_in, float* y,
                         void* y_bf16, void* stream);
int32_t ppf_sg_patch_bwd_weight(const PpfSgShape* s, const float* fields,
                                const void* dy_bf16, float* dw_in, float* db_in,
                                void* stream);
int32_t ppf_sg_block_fwd(const PpfSgShape* s, const float* y, const float* w_dw,
                         const float* b_dw, float* h, void* h_bf16,
                         const void* w1_bf16, const float* b1, float* pre,
                         void* act_bf16, const void* w2_bf16, const float* b2,
                         float* y_out, void* y_out_bf16, void* stream);
int32_t ppf_sg_block_bwd(const PpfSgShape* s, const float* y, const void* h_bf16,
                         const float* pre, const void* act_bf16,
                         const void* w1_bf16, const void* w2_bf16,
                         const float* w_dw, const float* dy_out,
                         const void* dy_out_bf16, void* dpre_bf16, float* dh,
                         void* dh_bf16, float* dy, float* dw1, float* db1,
                         float* dw2, float* db2, float* dw_dw, float* db_dw,
                         void* stream);
int32_t ppf_sg_head_fwd(const PpfSgShape* s, const void* y_bf16,
                        const void* w_out_bf16, const float* b_out, float* out,
                        void* stream);
int32_t ppf_sg_head_bwd(const PpfSgShape* s, const void* y_bf16,
                        const void* w_out_bf16, const void* dout_bf16,
                        float* dw_out, float* db_out, float* dy, void* dy_bf16,
                        void* stream);
/* loss += mean((out - (f_new - f_old) * s)^2); grad = d loss / d out (bf16) */
int32_t ppf_sg_mse(const PpfSgShape* s, const float* out, const float* f_old,
                   const float* f_new, void* grad_bf16, double* loss,
                   void* stream);
/* f_new = clamp(f_old + out / s, lo, hi) (the surrogate's k-step prediction) */
int32_t ppf_sg_apply(const PpfSgShape* s, const float* out, const float* f_old,
                     float* f_new, void* stream);
/* Window check: per sample b, out[3b] = sum_phi (k (stepped - pred) - (pred - u))^2,
 * out[3b+1] = sum_phi pred^2, out[3b+2] = cells with a non-finite pred or stepped. */
int32_t ppf_sg_residual(const PpfSgShape* s, const float* u, const float* pred,
                        const float* stepped, int32_t k, double* out, void* stream);
/* 1 (default): GEMMs whose operands are both K-contiguous, with at least 4096
 * rows, run on the tcgen05 tensor cores (accumulator in tensor memory);
 * 0: every GEMM on mma.sync. */
int32_t ppf_sg_set_tensor_path(int32_t tcgen05);
int32_t ppf_sg_cast_bf16(const float* x, void* y, long long n, void* stream);
int32_t ppf_sg_adam(float* w, void* w_bf16, const float* g, float* m1, float* m2,
                    long long n, float lr, float b1, float b2, float eps,
                    int32_t step, float weight_decay, void* stream);

/* ---- diagnostics (FP64 reductions) ------------------------------------ */

/* Bytes of caller-provided device scratch the reductions below need. */
int32_t ppf_reduce_scratch_bytes(const PpfGrid* g, size_t* bytes);
/* out[0] = sum of the interior cells in double (deterministic order):
 * the "mass" diagnostic. No counterpart in the reference (it has none). */
int32_t ppf_reduce_sum_f32(const float* x, const PpfGrid* g, double* out,
                           void* scratch, size_t scratch_bytes, void* stream);
int32_t ppf_reduce_sum_f64(const double* x, const PpfGrid* g, double* out,
                           void* scratch, size_t scratch_bytes, void* stream);
/* Same result as ppf_reduce_sum_f32, for callers that cannot allocate
 * device memory: a host application whose memory manager owns the whole
 * GPU, or code that is not allowed to call cudaMalloc (or any allocating
 * library routine) at the point where it needs the mass. It takes no
 * scratch argument and allocates nothing: its partial sums live in a fixed
 * 8 KiB device array inside the library (1024 doubles, one per first-pass
 * CTA; grids needing more are rejected with PPF_ERR_INVALID, which the
 * current split never does). The first call on each device looks up that
 * array's device address (cudaGetSymbolAddress) with the device current
 * (again after a context reset; concurrent host threads may make the first
 * call safely); make that first call before any stream capture. Every call
 * shares the
 * array, so calls that overlap on the GPU (different streams, or different
 * host threads, with no ordering between them) race and give wrong sums.
 * No counterpart in the reference. */
int32_t ppf_reduce_sum_f32_noalloc(const float* x, const PpfGrid* g, double* out,
                                   void* stream);
/* out[0] = dx^d * sum over cells of [w f(x) + kappa/2 |grad x|^2],
 * f(x) = x^2 (1-x)^2, forward differences with the boundary rule applied:
 * the free energy whose variation gives the Allen-Cahn (w = 16 W,
 * kappa = eps^2) and Cahn-Hilliard (w = 1, kappa = eps^2) updates. */
int32_t ppf_free_energy_f32(const float* x, const PpfGrid* g,
                            const PpfBoundary* bc, double dx, double w,
                            double kappa, double* out, void* scratch,
                            size_t scratch_bytes, void* stream);
int32_t ppf_free_energy_f64(const double* x, const PpfGrid* g,
                            const PpfBoundary* bc, double dx, double w,
                            double kappa, double* out, void* scratch,
                            size_t scratch_bytes, void* stream);
/* ORs PPF_STATUS_NONFINITE into *status (device memory) if any interior
 * cell is not finite: the NaN/Inf sentinel the engines run after every
 * chunk of steps. No counterpart in the reference (its engines never check). */
int32_t ppf_check_finite_f32(const float* x, const PpfGrid* g, int32_t* status,
                             void* stream);
int32_t ppf_check_finite_f64(const double* x, const PpfGrid* g, int32_t* status,
                             void* stream);

/* Reads and clears the library's device status word (PPF_STATUS_* bits
 * or'ed in by kernels: a bounded wait that gave up, a non-finite value).
 * Synchronous. */
int32_t ppf_status_take(int32_t* status);
/* Stream-ordered, graph-capturable form: moves the library's status bits
 * into *dst (device memory; *dst |= bits) and clears the library word, so
 * that an engine can keep its own sticky status word and copy it to the
 * host asynchronously. No counterpart in the reference. */
int32_t ppf_status_collect(int32_t* dst, void* stream);
/* Launches a kernel whose barrier wait can never complete, with a poll
 * limit, so that it gives up and reports PPF_STATUS_TIMEOUT (test of the
 * bounded-wait path; nothing is left in flight). */
int32_t ppf_selftest_wait_timeout(int32_t poll_limit, void* stream);

/* *counter += inc on the device (stream-ordered; one thread). */
int32_t ppf_counter_add_u64(uint64_t* counter, uint64_t inc, void* stream);

/* ---- CUDA graphs ------------------------------------------------------ */

/* Capture every launch issued on `stream` between begin and end into a
 * graph (the per-step Python loop of Simulation.simulate, simulation.py:
 * 262-271, replayed as one launch). */
int32_t ppf_graph_begin(void* stream);
int32_t ppf_graph_end(void* stream, void** graph_exec);
int32_t ppf_graph_launch(void* graph_exec, void* stream);
int32_t ppf_graph_destroy(void* graph_exec);

#ifdef __cplusplus
}
#endif

#endif /* PPF_GB300_H */
