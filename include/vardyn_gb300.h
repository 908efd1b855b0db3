/*
 * vardyn_gb300 — C ABI of the GB300 (sm_103a) backend for VarDyn's 4D-Var
 * inner loop: the QG 1.5-layer model step, its tangent-linear and adjoint,
 * the Helmholtz PV->SSH inversion and the along-track observation misfit.
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer unless its name ends in _host.
 *   - Fields are row-major [batch][ny][nx] (the reference's (ny, nx) State
 *     layout, mapping/src/state.py:52-56), contiguous, element type given by
 *     the plan's dtype (VD_F32 = float, VD_F64 = double).
 *   - Calls are stream-ordered on the caller's cudaStream_t (passed as void*),
 *     do not synchronise, do not allocate device memory (scratch comes in as a
 *     caller-owned workspace sized by the *_bytes queries), and return a
 *     vd_status. Plans own their constant tables (allocated once at create).
 *   - Batched calls advance `batch` independent windows of the same grid in
 *     lockstep; `batch` = 1 is the reference's single-window call.
 */
#ifndef VARDYN_GB300_H
#define VARDYN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int vd_status;
#define VD_OK 0
#define VD_ERR_ARG 1          /* bad dimension, null pointer, unknown option */
#define VD_ERR_CUDA 2         /* a CUDA runtime call failed */
#define VD_ERR_WORKSPACE 3    /* workspace smaller than the *_bytes query */
#define VD_ERR_UNSUPPORTED 4  /* grid too small/large for the kernels */
#define VD_ERR_SIZE 5         /* request larger than the fixed scratch of
                                 vd_qg1l_pv2h_noalloc */

#define VD_F32 0
#define VD_F64 1

/* Time schemes of Qgm.one_step (mapping/models/model_qg1l/jqgm.py:493-498);
 * VD_RK4 is an extension (classical Runge-Kutta 4), absent from Qgm. */
#define VD_EULER 0
#define VD_RK2 1
#define VD_RK3 2
#define VD_RK4 3

typedef struct vd_qg1l_plan vd_qg1l_plan;

/* Model constants, the arguments of Qgm.__init__
 * (mapping/models/model_qg1l/jqgm.py:113-236). */
typedef struct vd_qg1l_desc {
    int ny, nx;            /* grid shape (>= 8 each) */
    int dtype;             /* VD_F32 | VD_F64 */
    int time_scheme;       /* VD_EULER | VD_RK2 | VD_RK3 | VD_RK4 */
    double dx, dy;         /* grid spacing [m] (jqgm.py:126-131 centre value) */
    double dt;             /* time step [s] */
    double g;              /* gravity */
    double f;              /* Coriolis (nanmean of the f field, jqgm.py:140) */
    double c;              /* first baroclinic phase speed (jqgm.py:150-153) */
    double Kdiffus;        /* PV diffusion; used only if has_Kdiffus */
    int has_Kdiffus;
    const int8_t* mask_host;   /* [ny][nx] mask of jqgm.py:178-217 (0 land,
                                  1/2 rings, 3 interior); NULL = no land */
    const double* beta_host;   /* [ny][nx] beta at each T point, rows 1..ny-2
                                  used (jqgm.py:143,356-358); NULL = f-plane */
    const double* fbathy_host; /* [ny][nx] f*bathymetry_PV_term (jqgm.py:351-353);
                                  NULL = none */
    int dst_engine;            /* VD_DST_AUTO: tensor cores (tcgen05, 3xTF32)
                                  for float32 plans; VD_DST_FMA: CUDA-core FMA */
} vd_qg1l_desc;

#define VD_DST_AUTO 0
#define VD_DST_FMA 1

/* Launch schedule of a plan's Helmholtz inversion (x-DST pass, y tridiagonal
 * solve, inverse x-DST pass). Every field 0 keeps the built-in rule; the
 * autotuner (vardyn_gb300.autotune) times candidates and sets the fastest.
 * A schedule applies to launches issued after the call (a captured CUDA
 * graph keeps the schedule it was captured with); results agree to rounding
 * whatever the schedule. */
typedef struct vd_qg1l_schedule {
    int engine;          /* 0 rule (tensor cores for float32 plans built with
                            VD_DST_AUTO, else CUDA-core FMA / float64 FFT);
                            1 CUDA-core FMA; 2 tensor cores (float32 plans
                            built with VD_DST_AUTO) */
    int tc_group_fwd;    /* 32-column output tiles per CTA of the forward
                            tensor-core pass: 0 rule, or 1, 2, 4, 8 */
    int tc_group_inv;    /* the same for the inverse pass */
    int fma_rows;        /* rows per CTA of the FMA pass: 0 rule, 16, 32 or
                            64 (float32) */
    int tridiag_rows;    /* rows per thread of the tridiagonal solve: 0 rule,
                            8, 16 or 32 (used when the field fits, else the
                            rule) */
    int tridiag_lean;    /* 1: the float32 16-row tridiagonal kernel capped at
                            80 registers (three CTAs per SM instead of two);
                            0 the standard kernel */
    int stencil_loads;   /* tiles of the adjoint stage: 0 rule (bulk tensor
                            copies when nx is a multiple of 16 and the fields
                            are 16-byte aligned, else bounds-checked loads);
                            1 bounds-checked loads */
} vd_qg1l_schedule;

/* ------------------------------------------------------------------------
 * Overlapping-tile QG 1.5-layer model, forward (QgmWithTiles.step,
 * mapping/models/model_qg1l/jqgm.py:1033-1376). Every tile runs its own
 * QG1.5L model (tile-mean f and c, no beta or bathymetry, Dirichlet hb on
 * the tile edge) for nstep steps; the weighted tiles are blended. The tables
 * are device arrays the caller builds (the drop-in class does):
 * ------------------------------------------------------------------------ */
typedef struct vd_qgt_desc {
    int ny, nx;                 /* domain */
    int tile;                   /* tile side T (>= 8) */
    int ntiles;
    int dtype;                  /* VD_F32 | VD_F64 */
    int time_scheme;            /* VD_EULER | VD_RK2 */
    int has_Kdiffus;
    double dx, dy, dt, g, Kdiffus;  /* centre spacings of the domain (jqgm.py:126-128) */
    const int32_t* origins;     /* [ntiles][2] (row, column) of each tile, inside the domain */
    const double* f_tile;       /* [ntiles] tile means of f (jqgm.py:1313) */
    const double* c_tile;       /* [ntiles] tile means of c (jqgm.py:1314) */
    const int8_t* mask;         /* [ny][nx] classes of the domain mask (0 land, 1/2 rings, 3) */
    const void* S;              /* [T-2][T-2] orthonormal DST-I matrix */
    const void* lap;            /* [T-2][T-2] Laplacian eigenvalues of the tile (jqgm.py:1065-1067) */
    const void* weights;        /* [T][T] tile taper (jqgm.py:1069-1073) */
    const void* wsum;           /* [ny][nx] summed tapers */
    const void* mdt;            /* [ny][nx] or NULL */
} vd_qgt_desc;

/* Shared memory one tile needs (the tile kernel holds a whole tile); a step
 * is VD_ERR_UNSUPPORTED above 227 KiB (e.g. T = 64 fits in float32, T <= 48
 * in float64). */
size_t vd_qgt_shared_bytes(int tile, int dtype);
size_t vd_qgt_workspace_bytes(const vd_qgt_desc* desc);
/* h1 = QgmWithTiles.step(h0, hb, nstep), fields [ny][nx] in desc->dtype. */
vd_status vd_qgt_step(const vd_qgt_desc* desc, const void* h0, const void* hb, int nstep, void* h1,
                      void* work, size_t work_bytes, void* stream);
/* Tangent linear and adjoint of QgmWithTiles.step with respect to h0
 * (QgmWithTiles.step_tgl / step_adj, jqgm.py:1358-1376: jax.jvp / jax.vjp of
 * the blended step). dh1 = J dh0, adh0 = J^T adh1; land carries no
 * derivative and NaN in adh1 reads as 0. The workspace holds a slab per tile
 * and, for the adjoint, the stage inputs of every step of every tile (it grows
 * with nstep; adjoint != 0 sizes the adjoint's). The tile kernels keep only
 * the DST matrix, the eigenvalues and two work blocks in shared memory
 * (4 (T-2)^2 elements + T^2 bytes): T = 64 fits in both dtypes. */
size_t vd_qgt_ad_workspace_bytes(const vd_qgt_desc* desc, int nstep, int adjoint);
vd_status vd_qgt_step_tgl(const vd_qgt_desc* desc, const void* dh0, const void* h0, const void* hb, int nstep,
                          void* dh1, void* work, size_t work_bytes, void* stream);
vd_status vd_qgt_step_adj(const vd_qgt_desc* desc, const void* adh1, const void* h0, const void* hb, int nstep,
                          void* adh0, void* work, size_t work_bytes, void* stream);

/* ------------------------------------------------------------------------
 * QG 1.5-layer model with passive tracers, forward (Qgm_trac.step,
 * mapping/models/model_qg1l/jqgm.py:1551-2151). The SSH/PV part runs on a
 * vd_qg1l plan built without bathymetry (its dx, dy, dt, g, f, c, Kdiffus,
 * mask and beta); ntrac tracers per window are advected by the same
 * third-order upwind scheme, diffused with Kdiffus_trac, zeroed on land, and
 * after every step get boundary values (open boundaries of Mellor 1996 on
 * the edge, or the boundary field on the ring classes) and a relaxation to
 * the boundary field with weights wbc on rows/columns 1..n-2.
 * ------------------------------------------------------------------------ */
typedef struct vd_qgtrac_desc {
    int ntrac;              /* tracers per window (0: the SSH alone) */
    int time_scheme;        /* VD_EULER | VD_RK2 | VD_RK4 (classical Runge-Kutta 4:
                               the reference's rk4 for this class cannot run) */
    int advect_pv;          /* 0: the PV is only diffused (jqgm.py:1806-1815) */
    int bc_obc;             /* 1: open boundaries ('OBC'); 0: boundary values on the rings */
    int has_Kdiffus_trac;
    double Kdiffus_trac;
    const void* wbc;        /* [ny][nx] relaxation weights (plan dtype, device); needed when ntrac > 0 */
    const void* mdt;        /* [ny][nx] mean dynamic topography (plan dtype, device) or NULL */
} vd_qgtrac_desc;

size_t vd_qgtrac_workspace_bytes(const vd_qg1l_plan* plan, const vd_qgtrac_desc* desc, int batch);
/* nstep steps from SSH h0 [batch][ny][nx] and tracers c0 [batch][ntrac][ny][nx]
 * with boundary fields hb, cb of the same shapes (jqgm.py:2057-2139): h1 and
 * c1 are NaN on land, the MDT is added before and removed after. c0, cb, c1
 * may be NULL when ntrac = 0. */
vd_status vd_qgtrac_step(const vd_qg1l_plan* plan, const vd_qgtrac_desc* desc, int batch, const void* h0,
                         const void* c0, const void* hb, const void* cb, int nstep, void* h1, void* c1,
                         void* work, size_t work_bytes, void* stream);
/* Tangent linear and adjoint of vd_qgtrac_step with respect to (h0, c0)
 * (Qgm_trac.step_tgl / step_adj, jqgm.py:2141-2151: jax.jvp / jax.vjp of
 * step; hb, cb are not differentiated). Shapes of vd_qgtrac_step; the plan's
 * time scheme must be desc->time_scheme. tgl: (dh1, dc1) = J (dh0, dc0), zero
 * on land. adj: (adh0, adc0) = J^T (adh1, adc1), NaN in adh1 / adc1 read as 0.
 * The adjoint's workspace holds every stage input of every step (it grows
 * with nstep; adjoint != 0 sizes the adjoint's). */
size_t vd_qgtrac_ad_workspace_bytes(const vd_qg1l_plan* plan, const vd_qgtrac_desc* desc, int batch, int nstep,
                                    int adjoint);
vd_status vd_qgtrac_step_tgl(const vd_qg1l_plan* plan, const vd_qgtrac_desc* desc, int batch, const void* h0,
                             const void* c0, const void* hb, const void* cb, const void* dh0, const void* dc0,
                             int nstep, void* dh1, void* dc1, void* work, size_t work_bytes, void* stream);
vd_status vd_qgtrac_step_adj(const vd_qg1l_plan* plan, const vd_qgtrac_desc* desc, int batch, const void* h0,
                             const void* c0, const void* hb, const void* cb, const void* adh1, const void* adc1,
                             int nstep, void* adh0, void* adc0, void* work, size_t work_bytes, void* stream);

/* Build a plan: DST-I half matrices, tridiagonal multipliers, mask, beta and
 * bathymetry tables on the current device. Replaces the constant set-up of
 * Qgm.__init__ (jqgm.py:113-236). */
vd_status vd_qg1l_plan_create(vd_qg1l_plan** plan, const vd_qg1l_desc* desc);
vd_status vd_qg1l_plan_destroy(vd_qg1l_plan* plan);
/* VD_ERR_ARG for an out-of-range field, VD_ERR_UNSUPPORTED for a choice the
 * plan cannot run (tensor cores without its images, an FMA row tile above
 * the shared-memory limit). */
vd_status vd_qg1l_set_schedule(vd_qg1l_plan* plan, const vd_qg1l_schedule* schedule);
vd_status vd_qg1l_get_schedule(const vd_qg1l_plan* plan, vd_qg1l_schedule* schedule);

/* Workspace for one call of `batch` windows (forward, tangent, adjoint and
 * the solve all fit in it). */
size_t vd_qg1l_workspace_bytes(const vd_qg1l_plan* plan, int batch);
/* Trajectory storage of `nstep` steps: every stage state (h_s, q_s) of every
 * step plus the final state, as the adjoint needs them. */
size_t vd_qg1l_traj_bytes(const vd_qg1l_plan* plan, int batch, int nstep);
/* Index-free description of the trajectory layout: slot(n, s) = n*nstage+s,
 * each slot holds h then q, each [batch][ny][nx]. */
int vd_qg1l_nstage(const vd_qg1l_plan* plan);

/* SSH -> PV (Qgm.h2pv, jqgm.py:264-293). */
vd_status vd_qg1l_h2pv(const vd_qg1l_plan* plan, int batch, const void* h,
                       const void* hb, void* q, void* stream);
/* SSH -> geostrophic u, v (Qgm.h2uv, jqgm.py:238-262). */
vd_status vd_qg1l_h2uv(const vd_qg1l_plan* plan, int batch, const void* h,
                       void* u, void* v, void* stream);
/* PV tendency (Qgm.rhs, jqgm.py:321-375, way=+1). */
vd_status vd_qg1l_rhs(const vd_qg1l_plan* plan, int batch, const void* u,
                      const void* v, const void* q, void* rhs, void* stream);
/* PV -> SSH: h = L^-1(q - qb) on the interior + hb (Qgm.pv2h, jqgm.py:295-319,
 * inverse_elliptic_dst 83-91), by x-DST-I, y-tridiagonal solve, x-DST-I. */
vd_status vd_qg1l_pv2h(const vd_qg1l_plan* plan, int batch, const void* q,
                       const void* hb, const void* qb, void* h, void* work,
                       size_t work_bytes, void* stream);

/* PV -> SSH inversion that allocates nothing. No counterpart in the
 * reference: it exists for callers that cannot allocate GPU memory (code
 * inside a frozen CUDA-graph memory plan, plugins whose GPU memory belongs to
 * another allocator, FFI hosts that only pass buffers they own). Same result
 * as vd_qg1l_pv2h, but the spectral intermediate lives in a fixed array
 * compiled into the library (vd_qg1l_pv2h_noalloc_max_bytes(), 16 MiB; one
 * copy per device, held until the process exits): requests needing more
 * return VD_ERR_SIZE. The first call on a device looks up that array's
 * device address, so make it before capturing a stream. All calls share the
 * array: calls that may overlap on the GPU (other streams, other threads)
 * race on it and must be serialised by the caller. The device address is
 * cached per device ordinal for the life of the process, so a device reset
 * (cudaDeviceReset) while the library is loaded is not supported. */
size_t vd_qg1l_pv2h_noalloc_max_bytes(void);
vd_status vd_qg1l_pv2h_noalloc(const vd_qg1l_plan* plan, int batch, const void* q,
                               const void* hb, const void* qb, void* h,
                               void* stream);

/* The x-direction orthonormal DST-I of the solve alone (dstI1D along the
 * last axis, jqgm.py:75-77, applied to the (ny-2) x (nx-2) interior).
 * inverse == 0: field interior -> spec; inverse != 0: spec -> out interior.
 * spec rows hold the even wavenumbers (k = 0, 2, ...) first, then the odd
 * ones; its size is vd_qg1l_spec_bytes(plan, batch). */
size_t vd_qg1l_spec_bytes(const vd_qg1l_plan* plan, int batch);
/* The y-direction part of the solve alone, in place on spectral rows: for
 * every x-wavenumber k the tridiagonal system
 * g/f*(X[j-1] - 2X[j] + X[j+1])/dy^2 + (g/f*mu_k - g*f/c^2) X[j] = F[j]
 * with X = 0 beyond the walls (equal to the y-DST / eigenvalue division /
 * y-DST of inverse_elliptic_dst, jqgm.py:83-91). */
vd_status vd_qg1l_tridiag_y(const vd_qg1l_plan* plan, int batch, void* spec, void* stream);
/* inverse == 2 runs the inverse pass with the adjoint epilogue of the
 * solve: out = (mask == 3) ? x + field : 0 (field is the addend). */
vd_status vd_qg1l_dst_x(const vd_qg1l_plan* plan, int batch, const void* field,
                        void* spec, int inverse, void* out, void* stream);

/* One forward Runge-Kutta stage of Qgm.one_step (jqgm.py:480-503 with the
 * scheme bodies of 398-477): k = rhs(h2uv(hs), qs) (jqgm.py:238-262,
 * 321-396; 0 off the tendency points) and
 * q_out = q_base + sum_t c[t] * k_in[t] + c_self * k. k_in is a host array of
 * nk <= 4 device fields, c its host coefficients; k_out (nullable) receives
 * k. The kernel of the library's own steps, launched alone. */
vd_status vd_qg1l_rk_stage(const vd_qg1l_plan* plan, int batch, const void* hs,
                           const void* qs, const void* q_base, int nk,
                           const void* const* k_in, const double* c,
                           double c_self, void* k_out, void* q_out,
                           void* stream);
/* Adjoint of the tendency of one stage (the vjp of jqgm.py:238-262, 321-396
 * that step_adj takes through jax.vjp, jqgm.py:565-569): with the stage
 * cotangent lk = sum_t c[t] * g[t] on the tendency points, adh_out = the
 * SSH adjoint through h2uv, adq_out = (mask == 3) * (PV adjoint +
 * sum_t acc[t]). g (ng <= 4) and acc (nacc <= 4) are host arrays of device
 * fields, c host coefficients. */
vd_status vd_qg1l_rk_stage_adj(const vd_qg1l_plan* plan, int batch,
                               const void* hs, const void* qs, int ng,
                               const void* const* g, const double* c, int nacc,
                               const void* const* acc, void* adq_out,
                               void* adh_out, void* stream);

/* Forward model: Qgm.step (jqgm.py:517-557). h_out = M^nstep(h0) with
 * q0 = h2pv(h0, hb), land set to NaN. If traj != NULL (sized by
 * vd_qg1l_traj_bytes) every stage state is stored for a later adjoint.
 * h_out may alias h0. */
vd_status vd_qg1l_step(const vd_qg1l_plan* plan, int batch, const void* h0,
                       const void* hb, int nstep, void* h_out, void* traj,
                       void* work, size_t work_bytes, void* stream);
/* Tangent linear: Qgm.step_tgl (jqgm.py:559-563), dh_out = M'(h0) dh0. */
vd_status vd_qg1l_step_tgl(const vd_qg1l_plan* plan, int batch, const void* dh0,
                           const void* h0, const void* hb, int nstep,
                           void* dh_out, void* work, size_t work_bytes,
                           void* stream);
/* Adjoint: Qgm.step_adj (jqgm.py:565-569), adh_out = M'(h0)^T adh1.
 * traj must hold the trajectory of vd_qg1l_step(h0, hb, nstep); if
 * traj_ready == 0 it is recomputed into traj first. adh_out may alias adh1. */
vd_status vd_qg1l_step_adj(const vd_qg1l_plan* plan, int batch, const void* adh1,
                           const void* h0, const void* hb, int nstep,
                           void* adh_out, void* traj, int traj_ready,
                           void* work, size_t work_bytes, void* stream);

/* Lower-level state API used by the 4D-Var window engine: the state is the
 * pair (h, q) of Qgm.one_step (jqgm.py:480-503). */
/* q = h2pv(h, hb) and qb = h2pv(hb, hb) (jqgm.py:536-537). qlo (nullable,
 * [batch][ny][nx]): for float32 plans, the PV is evaluated in float64 and
 * returned as the unevaluated pair q + qlo, the start of a compensated state
 * (see vd_qg1l_advance). */
vd_status vd_qg1l_init_state(const vd_qg1l_plan* plan, int batch, const void* h,
                             const void* hb, void* q, void* qb, void* qlo,
                             void* stream);
/* nstep steps from traj slot (first_step*nstage) onwards; the starting state
 * must already be in that slot. Writes every stage slot and the slot of the
 * state after the last step. hb and qb may be NULL when the background SSH
 * is zero (then qb == 0 too); the solves then skip them.
 * qlo (nullable, [batch][ny][nx], updated in place): the low part of a
 * compensated PV state. The last stage of every step adds its increment to
 * the pair q + qlo with an error-free sum, so the roundings of a long window
 * do not accumulate in the trajectory (float32 plans; the library's own
 * steps always use it for float32 and never for float64, whose arithmetic
 * follows the reference's). NULL steps with plain arithmetic. */
vd_status vd_qg1l_advance(const vd_qg1l_plan* plan, int batch, void* traj,
                          int traj_steps, int first_step, int nstep,
                          const void* hb, const void* qb, void* qlo, void* work,
                          size_t work_bytes, void* stream);
/* Reverse of vd_qg1l_advance over the same steps: (adh, adq) holds the
 * adjoint of the state after step first_step+nstep-1 on entry and of the
 * state at first_step on exit. */
vd_status vd_qg1l_advance_adj(const vd_qg1l_plan* plan, int batch,
                              const void* traj, int traj_steps, int first_step,
                              int nstep, void* adh, void* adq, void* work,
                              size_t work_bytes, void* stream);
/* adh += h2pv'(h)^T adq (adjoint of jqgm.py:536, hb fixed). */
vd_status vd_qg1l_init_state_adj(const vd_qg1l_plan* plan, int batch,
                                 const void* h, const void* adq, void* adh,
                                 void* stream);
/* Output of a step call: land -> NaN, walls -> hb, plus coef*forcing if
 * forcing != NULL (jqgm.py:550-551 and mod.py:911-913). */
vd_status vd_qg1l_finalize(const vd_qg1l_plan* plan, int batch, const void* h,
                           const void* hb, const void* forcing, double coef,
                           void* h_out, void* stream);
/* vd_qg1l_finalize with one forcing coefficient per window: coef is a
 * DEVICE array of `batch` doubles (n*dt/86400 of each window's model call,
 * mod.py:911-913; 0 for a window that does not end a call here). */
vd_status vd_qg1l_force(const vd_qg1l_plan* plan, int batch, const void* h,
                        const void* hb, const void* forcing, const double* coef,
                        void* h_out, void* stream);
/* Adjoint of vd_qg1l_force: adforcing[b] += coef[b]*adh_out[b]
 * (mod.py:1058-1068) and adh = adh_out with the walls and land set to 0.
 * adh may alias adh_out. */
vd_status vd_qg1l_force_adj(const vd_qg1l_plan* plan, int batch, const void* adh_out,
                            void* adforcing, const double* coef, void* adh, void* stream);

/* Along-track observation operator (Obsop_interp_l3_jax, mapping/src/obsop.py
 * 375-678). H is stored per observation as up to 4 (grid index, weight) pairs
 * (index -1 = unused), already restricted to the valid neighbours of
 * _sparse_op (obsop.py:417-460). obs_field[o] selects which field of `fields`
 * (stride field_stride elements) observation o reads. */
/* misfit[o] = inverr[o] * (sum_m w[o,m] x[idx[o,m]] - y[o]), NaN -> 0
 * (obsop.py:610-628). */
vd_status vd_obs_misfit(int dtype, int nobs, const void* fields,
                        long long field_stride, const int32_t* obs_field,
                        const int32_t* idx4, const void* w4, const void* yobs,
                        const void* inverr, void* misfit, void* stream);
/* Adjoint (obsop.py:630-678): ad[field][g] += sum over the CSR list of grid
 * point g of w * inverr[o] * cot[o]. The CSR (rows = touched grid points,
 * entries = observation/weight pairs) is built once on the host. */
vd_status vd_obs_adjoint(int dtype, int npoints, void* ad_fields,
                         long long field_stride, const int32_t* pt_field,
                         const int32_t* pt_index, const int32_t* rowptr,
                         const int32_t* ent_obs, const void* ent_w,
                         const void* inverr, const void* cot, void* stream);

/* Deterministic FP64 reductions (Jo, Jb, gradient norms, dot-product test,
 * tools_4Dvar.py:265,292,326). nseg segments given by seg_off[nseg+1]. */
vd_status vd_sumsq_f64(int dtype, int nseg, const int32_t* seg_off,
                       const void* x, double* out, void* stream);
/* out[s] = scale * sum over k in [seg_off[s], seg_off[s+1]) of x[perm[k]]^2
 * (per-window Jo when observations are stored in time-major order). */
vd_status vd_sumsq_gather_f64(int dtype, int nseg, const int32_t* seg_off,
                              const int32_t* perm, const void* x, double scale,
                              double* out, void* stream);
/* out[0] = sum x*y in FP64; out must hold VD_DOT_SCRATCH doubles (the
 * partial sums live in out[1..]) so that the call allocates nothing. */
#define VD_DOT_SCRATCH 1025
vd_status vd_dot_f64(int dtype, long long n, const void* x, const void* y,
                     double* out, void* stream);
/* out[i] = d[i % period] * x[i] + (y ? y[i] : 0) for i < n (diagonal
 * covariance products of tools_4Dvar.py:28-45: X = Q X0 + Xb, G = Q adX + X0
 * over `batch` control vectors of length period). out may alias x or y. */
vd_status vd_diag_axpy(int dtype, long long n, long long period, const void* d,
                       const void* x, const void* y, void* out, void* stream);
/* y = a*x + b*y elementwise (n elements). */
vd_status vd_axpby(int dtype, long long n, double a, const void* x, double b,
                   void* y, void* stream);
/* y = x (n elements of the dtype); y = value. */
vd_status vd_copy(int dtype, long long n, const void* x, void* y, void* stream);
vd_status vd_fill(int dtype, long long n, double value, void* y, void* stream);

/* ------------------------------------------------------------------------
 * Gaussian space-time reduced basis (Basis_gauss3d, mapping/src/basis.py
 * 1170-1555; several components = Basis_multi, basis.py:4039-4135).
 *
 * The control vector X (nbasis coefficients per window) is the concatenation
 * over components c of [ENST_c.size][Nx_c] blocks (time centre major, space
 * centre minor, basis.py:1324,1441). At basis time k:
 *   phi = sum_c G_c(t_k) X_c,   G_c(t) X_c = Gauss_xy_c (sum_it g_it(t) X_c[it,:])
 * (operg, basis.py:1489-1524) and adX_c[it,:] += g_it(t_k) Gauss_xy_c^T adphi
 * (operg_transpose, basis.py:1526-1555). The grid must be rectilinear: x (or
 * longitude) depends on the column only and y (or latitude) on the row only.
 * ---------------------------------------------------------------------- */
typedef struct vd_basis_plan vd_basis_plan;

typedef struct vd_basis_grid {
    int ny, nx;
    int dtype;                  /* VD_F32 | VD_F64 of X and phi */
    int geographic;             /* 1: xc = longitude, yc = latitude in degrees
                                   (km2deg = 1/110, cos(lat) stretch, lon wrap:
                                   the reference's formulas); 0: x/y in km */
    const double* xc_host;      /* [nx] column coordinate */
    const double* yc_host;      /* [ny] row coordinate */
    const int8_t* land_host;    /* [ny][nx] nonzero = excluded point, or NULL */
    int ntime;                  /* basis times (days), the `time` argument */
    const double* time_host;    /*   of set_basis (basis.py:1291) */
    int host_only;              /* 1: build the tables on the host only, for
                                   the queries below (no device needed) */
} vd_basis_grid;

/* Parameters of one Basis_gauss3d component (config.BASIS, basis.py:1176-1187). */
typedef struct vd_gauss3d_params {
    double sigma_D;             /* space half-width [km] */
    double sigma_T;             /* time half-width [days] */
    double facns, facnlt;       /* space / time lattice densities */
    double sigma_Q;             /* prior std scale: Q = sigma_Q/sqrt(facns*facnlt) */
    int normalize_fact;         /* divide the time window by its integral */
    int flux;                   /* time window = mywindow_flux (basis.py:4142) */
    int has_time_spinup;
    double time_spinup;         /* [days], used if has_time_spinup */
} vd_gauss3d_params;

vd_status vd_basis_plan_create(vd_basis_plan** out, const vd_basis_grid* grid, int ncomp,
                               const vd_gauss3d_params* comps);
vd_status vd_basis_plan_destroy(vd_basis_plan* plan);
/* Total number of coefficients (sum over components of ENST.size * Nx). */
long long vd_basis_nbasis(const vd_basis_plan* plan);
/* Per component: offset of its block in X, number of time centres, number of
 * space centres. */
vd_status vd_basis_component(const vd_basis_plan* plan, int comp, long long* offset,
                             int* ntime_centres, int* nspace_centres);
/* Host copies of the lattice of one component: ENST [ntime_centres],
 * ENSLAT and ENSLON [nspace_centres] (basis.py:1304-1324); NULL skips one. */
vd_status vd_basis_lattice(const vd_basis_plan* plan, int comp, double* enst_host,
                           double* enslat_host, double* enslon_host);
/* Prior standard deviation of every coefficient [nbasis] (basis.py:1359). */
vd_status vd_basis_q(const vd_basis_plan* plan, double* q_host);
/* Active time centres of component comp at basis time k: their count, and
 * (it, weight) pairs if the arrays are non-NULL (at most the count). */
vd_status vd_basis_time_weights(const vd_basis_plan* plan, int k, int comp, int* count,
                                int* it_host, double* weight_host);
/* Workspace of vd_basis_project / vd_basis_project_T for `batch` windows. */
size_t vd_basis_workspace_bytes(const vd_basis_plan* plan, int batch);
/* phi[b] = (accumulate ? phi[b] : 0) + sum_c G_c(t_k) X[b] for b < batch;
 * X[b] starts at X + b*ldX, phi is [batch][ny][nx]; land points get 0. */
vd_status vd_basis_project(const vd_basis_plan* plan, int batch, int k, const void* X,
                           long long ldX, void* phi, int accumulate, void* workspace,
                           size_t workspace_bytes, void* stream);
/* adX[b] += G(t_k)^T adphi[b] over the coefficients active at t_k; adphi is
 * read only (the reference's zeroing of adState.params is the caller's). */
vd_status vd_basis_project_T(const vd_basis_plan* plan, int batch, int k, const void* adphi,
                             void* adX, long long ldX, void* workspace,
                             size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Wave-packet reduced basis (Basis_bm / Basis_bm_jax, mapping/src/basis.py
 * 472-1168) on a rectilinear grid given as for vd_basis_plan_create.
 * Frequencies ff between 1/lmax and 1/lmin, directions theta, per frequency
 * a lattice of centres and atoms sqrt(2) w(xx/DX) w(yy/DX) {cos, sin}(k.x);
 * the control vector holds, per frequency, [time centre][space centre]
 * [theta][cos, sin] coefficients (basis.py:775-781).
 * ---------------------------------------------------------------------- */
typedef struct vd_bm_plan vd_bm_plan;

typedef struct vd_bm_params {
    double npsp, facpsp;        /* wavelet extension / frequency step (basis.py:480-481) */
    double lmin, lmax;          /* wavelength range [km] */
    double facns, facnlt;       /* space / time lattice densities */
    double tdecmin, tdecmax;    /* decorrelation time bounds [days] */
    double factdec, sloptdec;   /* decorrelation time law (basis.py:651-656) */
    double Qmax, slopQ;         /* prior std law (basis.py:675-683) */
    double lmeso, tmeso;        /* mesoscale wavelength [km] and time [days] */
    int norm_time;              /* divide the time window by its integral */
    int flux;                   /* time window = mywindow_flux */
    double time_ref;            /* days from 1950-01-01 to the window start
                                   (delta_time_ref, basis.py:527) */
} vd_bm_params;

vd_status vd_bm_plan_create(vd_bm_plan** out, const vd_basis_grid* grid, const vd_bm_params* params);

/* Wavelet basis (Basis_wavelet3d, basis.py:2640-2985): the same atoms as the
 * wave packets, a lattice laid out from the domain centre, time centres of
 * every time frequency (Gaspari-Cohn windows) shared by all space
 * frequencies. The plan is a vd_bm_plan: every vd_bm_* query and projection
 * below applies (vd_bm_frequency's tdec is the first time scale). */
typedef struct vd_wavelet_params {
    double npsp, facpsp;        /* wavelet extension / frequency step (2647-2649) */
    double facnst;              /* lattice density in space and time */
    double lmin, lmax;          /* wavelength range [km] */
    double tmin, tmax;          /* period range [days] */
    double sigma_Q;             /* prior std of every coefficient */
} vd_wavelet_params;
vd_status vd_wavelet_plan_create(vd_bm_plan** out, const vd_basis_grid* grid,
                                 const vd_wavelet_params* params);
/* Wave packets with per-location decorrelation times and variances
 * (Basis_bmaux / Basis_bmaux_jax, basis.py:1741-2638): the atoms and the
 * lattice of the wave packets (the lattice ends at LAT_MAX + DX, LON_MAX +
 * DX/cos), but every space centre P of a frequency takes its decorrelation
 * time (factdec * the mean of Tdec over a 10 x 10 grid of its box, clipped),
 * window integral and time centres (from -time_ref mod tdec, spaced
 * tdec / facnlt) of its own, and Q = facQ * the box mean of Std; a
 * frequency's time axis is padded to its longest list (padded centres have
 * weight 0 and Q = 1e-10 facQ). The auxiliary fields are host arrays
 * [aux_nf][aux_nlat][aux_nlon] on ascending coordinates in the grid's
 * longitude convention, interpolated as xarray's DataArray.interp with 1-D
 * indexers does (orthogonal points, linear, NaN outside). Controls of one
 * frequency are ordered [time centre][space centre][theta][cos, sin]. Every
 * vd_bm_* query and projection applies, except vd_bm_time_weights (the time
 * weights are per centre); vd_bm_frequency's tdec is 0 and its time-centre
 * count the padded one; vd_bm_lattice's enst is [NP][padded count] (NaN
 * padding). */
typedef struct vd_bmaux_params {
    double npsp, facpsp, lmin, lmax, facns, facnlt;
    double tdecmin, tdecmax, factdec;   /* decorrelation time bounds and factor */
    double facQ;                        /* factor of the prior std */
    int norm_time, flux;
    double time_ref;                    /* days from 1950-01-01 to the window start */
    int aux_nf, aux_nlat, aux_nlon;     /* auxiliary grid (each >= 2) */
    const double *aux_f, *aux_lat, *aux_lon;   /* ascending coordinates */
    const double *aux_tdec, *aux_std;          /* [aux_nf][aux_nlat][aux_nlon], NaN allowed */
} vd_bmaux_params;
vd_status vd_bmaux_plan_create(vd_bm_plan** out, const vd_basis_grid* grid, const vd_bmaux_params* params);
/* Per space centre of frequency iff: decorrelation time, window integral and
 * number of time centres (any pointer may be NULL). */
vd_status vd_bmaux_centres(const vd_bm_plan* plan, int iff, double* tdec_host, double* norm_host, int* nt_host);
vd_status vd_bm_plan_destroy(vd_bm_plan* plan);
long long vd_bm_nbasis(const vd_bm_plan* plan);
/* Number of frequencies and directions; theta_host [ntheta] if non-NULL. */
vd_status vd_bm_shape(const vd_bm_plan* plan, int* nf, int* ntheta, double* theta_host);
/* Per frequency: ff [1/km], tdec [days], offset of its block in X, number of
 * time centres and of space centres (any pointer may be NULL). */
vd_status vd_bm_frequency(const vd_bm_plan* plan, int iff, double* ff, double* tdec,
                          long long* offset, int* ntime_centres, int* nspace_centres);
vd_status vd_bm_lattice(const vd_bm_plan* plan, int iff, double* enst_host,
                        double* enslat_host, double* enslon_host);
vd_status vd_bm_q(const vd_bm_plan* plan, double* q_host);
vd_status vd_bm_time_weights(const vd_bm_plan* plan, int k, int iff, int* count,
                             int* it_host, double* weight_host);
size_t vd_bm_workspace_bytes(const vd_bm_plan* plan, int batch);
/* phi[b] = (accumulate ? phi[b] : 0) + G(t_k) X[b]; adX[b] += G(t_k)^T adphi[b]. */
vd_status vd_bm_project(const vd_bm_plan* plan, int batch, int k, const void* X, long long ldX,
                        void* phi, int accumulate, void* workspace, size_t workspace_bytes,
                        void* stream);
vd_status vd_bm_project_T(const vd_bm_plan* plan, int batch, int k, const void* adphi,
                          void* adX, long long ldX, void* workspace, size_t workspace_bytes,
                          void* stream);

/* ------------------------------------------------------------------------
 * Masked multigrid Helmholtz solver (MG_Helmholtz,
 * mapping/models/model_qgsw/helmholtz_multigrid.py:156-419):
 *   div(c grad u) - lambda_b u = rhs_b  for b < nsys
 * on cell centres of an n0 x n1 rectangle (row-major [nsys][n0][n1]; axis 0
 * has spacing d0, axis 1 spacing d1), mask 1 inside / 0 outside, homogeneous
 * Neumann walls on cell edges. Full-multigrid start then max_ite V-cycles of
 * 6-sweep damped Jacobi smoothing; bottom solve by pseudo-inverse
 * (niter_bottom <= 0) or niter_bottom Jacobi smooths.
 * ---------------------------------------------------------------------- */
typedef struct vd_mg_plan vd_mg_plan;

typedef struct vd_mg_desc {
    int n0, n1;                 /* grid; both divisible by 2^(n_levels-1) */
    int nsys;                   /* systems solved together */
    int dtype;                  /* VD_F32 | VD_F64 */
    double d0, d1;              /* cell sizes along axis 0 and axis 1 */
    const double* lambda_host;  /* [nsys] */
    const double* mask_host;    /* [n0][n1], or NULL (no mask) */
    const double* coef_u_host;  /* [n0+1][n1] coefficient on axis-0 edges */
    const double* coef_v_host;  /* [n0][n1+1] coefficient on axis-1 edges */
    int n_levels;               /* 0: compute_nlevels (helmholtz_multigrid.py:27-33) */
    int max_ite;                /* final V-cycles (the reference's default is 20) */
    int niter_bottom;           /* <= 0: pseudo-inverse bottom solve */
} vd_mg_desc;

vd_status vd_mg_plan_create(vd_mg_plan** out, const vd_mg_desc* desc);
vd_status vd_mg_plan_destroy(vd_mg_plan* plan);
int vd_mg_levels(const vd_mg_plan* plan);
size_t vd_mg_workspace_bytes(const vd_mg_plan* plan);
/* f = FMG_Helmholtz(rhs) (helmholtz_multigrid.py:380-419). The first solve
 * with a given workspace captures the whole solve as a CUDA graph on
 * plan-owned rhs / solution buffers; later solves copy rhs in, replay it and
 * copy f out, so solves on one plan must not run concurrently (one stream at
 * a time). Called while the caller's stream is capturing, it launches the
 * kernels directly into the caller's graph. */
vd_status vd_mg_solve(const vd_mg_plan* plan, const void* rhs, void* f, void* workspace,
                      size_t workspace_bytes, void* stream);
/* res = rhs - H f on the finest level (helmholtz_multigrid.py:102-114). */
vd_status vd_mg_residual(const vd_mg_plan* plan, const void* f, const void* rhs, void* res,
                         void* stream);

/* ------------------------------------------------------------------------
 * Masked Dirichlet multigrid for the PV inversion of the multilayer QG
 * model on a domain with land (mapping/models/model_qgsw/qg.py:222-298, the
 * problem the reference solves with a DST and a capacitance-matrix
 * correction, helmholtz.py:146-184): per mode m, on n0 x n1 interior psi
 * nodes, (u_E + u_W - 2u)/d0^2 + (u_N + u_S - 2u)/d1^2 - lambda_m u = b at
 * nodes with mask != 0, u = 0 at masked nodes and beyond the boundary.
 * Node-centred geometric V-cycles (red-black Gauss-Seidel, full weighting,
 * bilinear prolongation) preconditioning conjugate gradients, the coarsest
 * level solved with a float64 inverse;
 * a solve stops each system at ||b - A u|| <= tol ||b|| (float64 norms) or
 * after max_cycles. No counterpart class in the reference.
 * ------------------------------------------------------------------------ */
typedef struct vd_mgd_plan vd_mgd_plan;
typedef struct vd_mgd_desc {
    int n0, n1;                 /* interior nodes; coarsening needs n+1 even */
    int nmode;                  /* systems per batch entry (vertical modes) */
    int dtype;                  /* VD_F32 | VD_F64 */
    double d0, d1;              /* node spacings */
    const double* lambda_host;  /* [nmode] */
    const double* mask_host;    /* [n0][n1], 0 = land (Dirichlet 0); NULL: none */
    int max_cycles;             /* conjugate-gradient iterations at most */
    double tol;                 /* relative residual that stops a system */
} vd_mgd_desc;
vd_status vd_mgd_plan_create(vd_mgd_plan** out, const vd_mgd_desc* desc);
vd_status vd_mgd_plan_destroy(vd_mgd_plan* plan);
int vd_mgd_levels(const vd_mgd_plan* plan);
int vd_mgd_coarse_unknowns(const vd_mgd_plan* plan);
size_t vd_mgd_workspace_bytes(const vd_mgd_plan* plan, int batch);
/* u = A^-1 b for batch * nmode systems, system s = m * batch + k using
 * lambda_m; element (i, j) of system s at b[s * fsb + i * ldb + j] (and the
 * same for u with ldu / fsu), so the interior of a padded field is solved in
 * place. rel (device, nullable): [batch * nmode] relative residual reached. */
vd_status vd_mgd_solve(const vd_mgd_plan* plan, int batch, const void* b, long long ldb,
                       long long fsb, void* u, long long ldu, long long fsu, double* rel,
                       void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Spectral Helmholtz helpers (mapping/models/model_qgsw/helmholtz.py). The
 * DST-I solve of one mode, div grad u - s u = rhs with Dirichlet walls
 * (solve_helmholtz_dstI, 138-143), is vd_qg1l_pv2h of a plan built with
 * g = f = 1 and c = 1/sqrt(s) on the (n0+1) x (n1+1) field.
 * ---------------------------------------------------------------------- */
/* dst[f][i][j] = src[f][clamp(i, 1, n0-2)][clamp(j, 1, n1-2)] * mask[i][j]
 * for nfield [n0][n1] fields: the walls take the nearest interior value
 * (jnp.pad mode='edge'), then the optional [n0][n1] mask multiplies. In place
 * (src == dst) only without a mask. */
vd_status vd_edge_pad(int dtype, int nfield, int n0, int n1, const void* src,
                      const void* mask, void* dst, void* stream);
/* Transpose of vd_edge_pad (mask applied first): the interior of out
 * [n0][n1] gathers from every position that copies it; walls are zero.
 * out must not alias ad. */
vd_status vd_edge_pad_adj(int dtype, int nfield, int n0, int n1, const void* ad,
                          const void* mask, void* out, void* stream);
/* Capacitance correction of solve_helmholtz_dstI_cmm (172-184) for nsys
 * systems of nper fields each (field f = s * nper + r, system-major):
 * out = rhs, then out[f][bidx[i]] += sum_j cap[s][i][j] * (-sol[f][bidx[j]])
 * for the M irregular-boundary points bidx (flat indices into a field of
 * field_elems elements; cap is [nsys][M][M]). out may alias rhs, not sol. */
vd_status vd_cmm_correct(int dtype, int nsys, int nper, int M, long long field_elems,
                         const void* cap, const int32_t* bidx, const void* sol,
                         const void* rhs, void* out, void* stream);

/* ------------------------------------------------------------------------
 * Spectral Helmholtz solve with Neumann boundaries on a rectangular domain
 * (mapping/models/model_qgsw/helmholtz.py HelmholtzNeumannSolver, 187-303,
 * on an all-ocean mask: the solve is its G alone, solve_helmholtz_dctII
 * 81-87). Fields are [nfield][nx][ny], y contiguous.
 * ---------------------------------------------------------------------- */
typedef struct vd_neumann_plan vd_neumann_plan;
/* HelmholtzNeumannSolver(nx, ny, dx, dy, lambd, dtype) (187-225): the
 * operator's DCT-II eigenvalues compute_laplace_dctII(nx, ny, dx, dy) -
 * lambd (22-30) at every point of [nx][ny], dx and dy scalars (element [0])
 * or [nx][ny] fields (dxy_spatial != 0), lambd a scalar or a [nx][ny] field
 * (lambd_spatial != 0), as the reference broadcasts them. VD_ERR_UNSUPPORTED
 * when a transform does not fit shared memory (nx or ny above 6400 in
 * float64, 12800 in float32), VD_ERR_ARG for a zero or non-finite
 * eigenvalue. */
vd_status vd_neumann_plan_create(vd_neumann_plan** out, int nx, int ny, int dtype,
                                 const double* dx_host, const double* dy_host, int dxy_spatial,
                                 const double* lambd_host, int lambd_spatial);
void vd_neumann_plan_destroy(vd_neumann_plan* plan);
/* HelmholtzNeumannSolver.solve (296-303): out = idctII2D(dctII2D(rhs) /
 * helm) (unnormalised DCT-II pair along each axis, 33-78) for nfield fields
 * of the plan's dtype; out may equal rhs. No workspace. */
vd_status vd_neumann_solve(const vd_neumann_plan* plan, int nfield, const void* rhs, void* out,
                           void* stream);

/* ------------------------------------------------------------------------
 * Multilayer rotating shallow-water model (mapping/models/model_qgsw/sw.py
 * SW with masks.py, flux.py, reconstruction.py, finite_diff.py).
 * Layout is the reference's: [batch][layer][x][y], y contiguous; u fields
 * are [nx+1][ny], v fields [nx][ny+1], h fields [nx][ny]. Step inputs and
 * outputs are physical fields (SW.step, sw.py:752-904).
 * ---------------------------------------------------------------------- */
typedef struct vd_sw_plan vd_sw_plan;

typedef struct vd_sw_desc {
    int nx, ny, nl;               /* nl <= 8 */
    int dtype;                    /* VD_F32 / VD_F64 */
    const double* dx_host;        /* [nx][ny] metric terms (sw.py:142-167) */
    const double* dy_host;        /* [nx][ny] */
    const double* f_host;         /* [nx+1][ny+1] Coriolis on the vorticity grid */
    const double* H_host;         /* [nl] or, with H_spatial, [nl][nx][ny] */
    int H_spatial;
    const double* g_prime_host;   /* [nl] */
    const double* mask_host;      /* [nx][ny] 0/1 ocean mask, NULL = all ocean */
    double slip_coef;             /* 1 free slip, 0 no slip */
    double bottom_drag_coef;
    double rho_water;             /* <= 0: 1025 */
    double h_min;                 /* minimum thickness of smooth_clamp (0.1) */
    double h_min_sharpness;       /* <= 0: 10 */
    double visc_coef, diff_coef;
    double dt;
    double sponge_coef;
    int flag_linear;
    int forcing_momentum;         /* 0 'direct', 1 'mass_consistent' */
    int h_wind_mode;              /* 0 none (reference thickness), 1 scalar, 2 field */
    double h_wind_scalar;
    const double* h_wind_host;    /* [nx][ny] */
    double taux_scalar, tauy_scalar;
    const double* taux_host;      /* [nx-1][ny] or NULL (scalar) */
    const double* tauy_host;      /* [nx][ny-1] or NULL (scalar) */
    const double* sponge_u_host;  /* [nx+1][ny] or NULL */
    const double* sponge_v_host;  /* [nx][ny+1] or NULL */
    const double* sponge_h_host;  /* [nx][ny] or NULL */
    const double* Hwind_host;     /* h_wind_mode 0: the layer-0 thickness [nx][ny] the wind
                                     depth is taken from (sw.py:622-630 read the model's
                                     own H, not a perturbed one); NULL = this plan's H */
    int barotropic_filter;        /* 0 off; 1 the spectral barotropic filter of every
                                     right-hand side (sw.py:305-320, 720-750): an
                                     all-ocean mask only (VD_ERR_UNSUPPORTED otherwise, as
                                     the reference's solver does not construct with land) */
    const double* bf_lambd_host;  /* the filter's lambd = 1 / (g' dt tau H_tot)
                                     (sw.py:316-317, the model's own H, not a perturbed
                                     one): a scalar or, with bf_lambd_spatial, [nx][ny];
                                     NULL = from this plan's H */
    int bf_lambd_spatial;
    int flag_obc;                 /* open boundaries (sw.py:353-371): the u masks of the
                                     west / east faces and the v masks of the south /
                                     north faces are 1 (set after the stencil masks are
                                     built); inflow velocities there are kept */
} vd_sw_desc;

/* Host-only: the flag bytes of the staggered masks (masks.py:57-158).
 * fh [nx][ny] bit0 mask_h; fu [nx+1][ny] bit0 mask_u, bits 1-3 h-stencil
 * eq2/eq4/gt6 along x, bits 4-6 w-stencil eq2/eq4/gt4 along y; fv
 * [nx][ny+1] bit0 mask_v, bits 1-3 h-stencil along y, bits 4-6 w-stencil
 * eq2/eq4/gt6 along x; fw [nx+1][ny+1] bits valid, cornerout, vertical,
 * horizontal boundary, w, psi. Any output may be NULL. */
vd_status vd_sw_masks(int nx, int ny, const double* mask, uint8_t* fh, uint8_t* fu,
                      uint8_t* fv, uint8_t* fw);
vd_status vd_sw_plan_create(vd_sw_plan** out, const vd_sw_desc* desc);
void vd_sw_plan_destroy(vd_sw_plan* plan);
size_t vd_sw_workspace_bytes(const vd_sw_plan* plan, int batch, int nstep);
/* Cotangents of H and h_wind (the H / h_wind entries of jax.vjp in
 * sw.py:924-938 and mod.py:3255-3290). While a zeroed buffer of
 * vd_sw_ref_adj_bytes is registered with vd_sw_set_ref_adj, every adjoint
 * call on the plan accumulates into it the cotangents of the tables built
 * from H and h_wind (reference thickness on h / u / v points, reference
 * pressure gradients, wind factors), summed over batch, stages and steps;
 * register NULL to stop. vd_sw_ref_pullback maps the buffer to adH
 * [nl][nx][ny] (the cotangent of every layer's thickness H, sw.py:386-406)
 * and, when adhw is not NULL, to the cotangent of a field h_wind [nx][ny]
 * (zero unless the plan's h_wind is a field, sw.py:608-640). Registration is
 * plan state: one adjoint at a time per plan. */
size_t vd_sw_ref_adj_bytes(const vd_sw_plan* plan);
vd_status vd_sw_set_ref_adj(vd_sw_plan* plan, void* buf);
vd_status vd_sw_ref_pullback(const vd_sw_plan* plan, const void* buf, void* adH, void* adhw,
                             void* stream);
/* Tangent with respect to H and h_wind (the dH / dh_wind inputs of the jvp
 * of SW.step, sw.py:906-922, used by Model_qgsw.jstep_tgl, mod.py:3222-3253):
 * computes the tangents of the H / h_wind dependent tables (reference
 * thickness and its face averages, reference pressure gradients; the wind
 * factors move only with h_wind, the wind depth of a perturbed H being the
 * model's own) on the host and registers them for the following
 * vd_sw_step_tgl / vd_sw_rhs_tgl calls. dH_host [nl][nx][ny] and
 * dhwind_host [nx][ny] (a scalar h_wind plan reads dhwind_host[0]) may be
 * NULL; buf is a device buffer of vd_sw_ref_adj_bytes(plan) bytes that stays
 * alive while registered; buf NULL unregisters. Synchronous (one host to
 * device copy). */
vd_status vd_sw_set_ref_tangent(vd_sw_plan* plan, const double* dH_host, const double* dhwind_host, void* buf);
/* nstep RK3-SSP steps. ub/vb/hb (sponge targets) default to the initial
 * state, Fu/Fv/Fh (forcing) to zero, taux [nx-1][ny] / tauy [nx][ny-1] to
 * the plan's wind stress; all are physical, all nullable (in groups of
 * three). */
vd_status vd_sw_step(vd_sw_plan* plan, int batch, const void* u0, const void* v0,
                     const void* h0, int nstep, const void* ub, const void* vb,
                     const void* hb, const void* Fu, const void* Fv, const void* Fh,
                     const void* taux, const void* tauy, void* u1, void* v1, void* h1,
                     void* work, size_t work_bytes, void* stream);
/* Tangent linear of vd_sw_step (jax.jvp, sw.py:906-922) in the initial state
 * and, optionally, the sponge targets and the forcing. */
vd_status vd_sw_step_tgl(vd_sw_plan* plan, int batch, const void* u0, const void* v0,
                         const void* h0, const void* du0, const void* dv0, const void* dh0,
                         int nstep, const void* ub, const void* vb, const void* hb,
                         const void* dub, const void* dvb, const void* dhb,
                         const void* Fu, const void* Fv, const void* Fh,
                         const void* dFu, const void* dFv, const void* dFh,
                         const void* taux, const void* tauy, void* du1, void* dv1,
                         void* dh1, void* work, size_t work_bytes, void* stream);
/* Adjoint of vd_sw_step (jax.vjp, sw.py:924-938): overwrites adu0/adv0/adh0;
 * writes the adjoints of the sponge targets and of the forcing when asked
 * (when the targets default to the initial state their adjoint is part of
 * adu0/adv0/adh0). No atomics on the state and forcing cotangents: repeated
 * runs agree bit for bit. The H / h_wind table cotangents of a registered
 * vd_sw_set_ref_adj buffer are summed over the batch with atomics (bit for
 * bit for batch 1, to rounding otherwise). */
vd_status vd_sw_step_adj(vd_sw_plan* plan, int batch, const void* u0, const void* v0,
                         const void* h0, const void* adu1, const void* adv1,
                         const void* adh1, int nstep, const void* ub, const void* vb,
                         const void* hb, const void* Fu, const void* Fv, const void* Fh,
                         const void* taux, const void* tauy, void* adu0, void* adv0,
                         void* adh0, void* adub, void* advb, void* adhb, void* adFu,
                         void* adFv, void* adFh, void* work, size_t work_bytes,
                         void* stream);
/* compute_time_derivatives (sw.py:720-750) of model-space fields (u dx,
 * v dy, h area), without sponge. */
vd_status vd_sw_rhs(vd_sw_plan* plan, int batch, const void* u, const void* v,
                    const void* h, const void* taux, const void* tauy, void* du, void* dv,
                    void* dh, void* work, size_t work_bytes, void* stream);

/* Shallow-water building blocks for drivers that insert an operator between
 * the right-hand side and the RK3-SSP combination (the QG model projects
 * every tendency). All fields are model-space (u dx, v dy, h area).
 * vd_sw_rhs_tgl: right-hand side and its tangent. vd_sw_rhs_adj: adds the
 * transpose of the right-hand side's Jacobian at (u, v, h) applied to
 * (aku, akv, akh) into (adu, adv, adh). */
vd_status vd_sw_rhs_tgl(vd_sw_plan* plan, int batch, const void* u, const void* v,
                        const void* h, const void* du, const void* dv, const void* dh,
                        const void* taux, const void* tauy, void* ku, void* kv, void* kh,
                        void* dku, void* dkv, void* dkh, void* work, size_t work_bytes,
                        void* stream);
vd_status vd_sw_rhs_adj(vd_sw_plan* plan, int batch, const void* u, const void* v,
                        const void* h, const void* aku, const void* akv, const void* akh,
                        void* adu, void* adv, void* adh, void* work, size_t work_bytes,
                        void* stream);
/* One RK3-SSP stage (sw.py:831-877): fields[24] = x(u,v,h), rhs, k0, k1,
 * sponge target, forcing (nullable; added at stage 2), k_out (stages 0, 1),
 * next. k = rhs + sponge rate * (target - x). */
vd_status vd_sw_stage(vd_sw_plan* plan, int batch, int stage, const void* const* fields,
                      void* stream);
/* Transpose of vd_sw_stage: fields[15] = adjoint of next (in place: becomes
 * the direct adjoint of x), adk out, adk0 / adk1 accumulators, sponge-target
 * adjoint accumulator. */
vd_status vd_sw_stage_adj(vd_sw_plan* plan, int batch, int stage, void* const* fields,
                          void* stream);
/* physical <-> model space: to_physical = 0 masks and multiplies by the
 * metrics (set_input_uvh), 1 divides (get_physical_uvh). Nullable fields. */
vd_status vd_sw_scale(vd_sw_plan* plan, int batch, int to_physical, const void* u,
                      const void* v, const void* h, void* uo, void* vo, void* ho,
                      void* stream);
/* mass-consistent forcing (sw.py:880-898): fields[9] = x, F, out; its
 * transpose: fields[8] = u, v, h, Fh, adu, adv (in place), adh (+=), adFh
 * (+=, nullable). */
vd_status vd_sw_force_mc(vd_sw_plan* plan, int batch, const void* const* fields, void* stream);
vd_status vd_sw_force_mc_adj(vd_sw_plan* plan, int batch, const void* const* fields,
                             void* stream);

/* ------------------------------------------------------------------------
 * QG projector of the multilayer QG model (mapping/models/model_qgsw/qg.py:
 * G 198-219, QoG_inv 222-298, Q 300-308) around the spectral Helmholtz
 * solves. Uniform dx, dy (the reference's QG operators need scalars).
 * ---------------------------------------------------------------------- */
typedef struct vd_qgp_plan vd_qgp_plan;
typedef struct vd_qgp_desc {
    int nx, ny, nl, dtype;
    double dx, dy, f0;
    const double* H_host;      /* [nl] */
    const double* A_host;      /* [nl][nl] layer coupling (qg.py:45-59) */
    const double* Cl2m_host;   /* [nl][nl] layer -> mode */
    const double* Cm2l_host;   /* [nl][nl] mode -> layer */
    const double* mask_host;   /* [nx][ny] h mask, NULL = all ocean */
    int cmm;                   /* 1: multiply the modal right-hand side by psi */
} vd_qgp_desc;
vd_status vd_qgp_plan_create(vd_qgp_plan** out, const vd_qgp_desc* desc);
void vd_qgp_plan_destroy(vd_qgp_plan* plan);
/* op 0 Q (u, v, h -> modes [nl][batch][nx+1][ny+1], walls 0); 1 its
 * transpose (modes -> adu, adv, adh); 2 per-field float64 sums (x, weights
 * [nl][nx+1][ny+1] or NULL, out: nl*batch sums followed by nl*batch*64
 * partials of scratch); 3 modal solutions, their sums,
 * homsol means [nl] (float64) and homsol -> p_qg [batch][nl][nx+1][ny+1];
 * 4 transpose of the mode -> layer mixing; 5 transpose of the homogeneous
 * correction (sums of homsol * ad, means, ad in place); 6 G (p_qg -> u, v,
 * h); 7 its transpose. */
vd_status vd_qgp_op(const vd_qgp_plan* plan, int op, int batch, const void* const* args,
                    void* stream);

/* Observation-operator construction on the device (obsop.py:417-460): for
 * each of nobs planar positions (km) the npix <= 4 nearest points of the
 * uniform (ny, nx) grid with spacing dx_km, dy_km (point (i, j) at (i dx,
 * j dy)), neighbours beyond dmax_km dropped (index -1, weight 0), Gaussian
 * weights exp(-D^2 / (2 (dmax/2)^2)) normalised per observation (npix = 1:
 * weight 1). idx [nobs][4] = j * nx + i, w [nobs][4] (float64). Ties in
 * distance go to the smaller index. */
vd_status vd_obs_knn(long long nobs, const double* x_km, const double* y_km, int ny, int nx,
                     double dx_km, double dy_km, int npix, double dmax_km, long long* idx,
                     double* w, void* stream);
/* vd_obs_knn with the neighbour rules of the scipy operator Obsop_interp_l3
 * (obsop.py:197-219): exclude [ny * nx] bytes (device, nullable), nonzero
 * for grid points that may not carry a weight (its ind_borders and ind_mask,
 * obsop.py:118-134). An excluded point keeps its place among the npix
 * nearest and gets index -1, weight 0; the kept weights are normalised over
 * the kept points. exclude = NULL is vd_obs_knn. */
vd_status vd_obs_knn_excl(long long nobs, const double* x_km, const double* y_km, int ny, int nx,
                          double dx_km, double dy_km, int npix, double dmax_km,
                          const unsigned char* exclude, long long* idx, double* w, void* stream);

/* ------------------------------------------------------------------------
 * Batched float64 vector kernels of the outer minimisation (L-BFGS without
 * bounds for batch independent windows, mapping/src/inv.py:309-414):
 * arrays are [batch][n]; coefficients are per-window device arrays so the
 * two-loop recursion needs no host round trip.
 * ---------------------------------------------------------------------- */
size_t vd_bdot_workspace_bytes(int batch, long long n);
/* out[b] = c0[b] + c1[b] * (x[b] . y[b]); c0 / c1 nullable (0 / 1);
 * deterministic (fixed reduction order). */
vd_status vd_bdot_f64(int batch, long long n, const double* x, const double* y,
                      const double* c0, const double* c1, double* out, void* work,
                      size_t work_bytes, void* stream);
/* y[b] = beta * y[b] + scale * coef[b] * x[b]; coef nullable (1). */
vd_status vd_baxpy_f64(int batch, long long n, double scale, const double* coef,
                       const double* x, double beta, double* y, void* stream);
/* z[b] = x[b] + coef[b] * y[b] */
vd_status vd_bxpay_f64(int batch, long long n, const double* x, const double* coef,
                       const double* y, double* z, void* stream);

/* Version / build information string. */
const char* vd_version(void);
/* Number of kernels this library has launched in the process so far (also
 * counts launches recorded into a CUDA graph during capture). */
long long vd_launch_count(void);
/* Device-side error bits set by bounded waits that ran out (1: stage
 * recycle, 2: operand arrival, 4: accumulator completion, 16: the peer
 * CTA's half tile of the inverse pass, of the tensor-core DST; 8: the staged
 * tiles of the QG adjoint stage); 0 = none.
 * Synchronous; reset != 0 clears them. */
vd_status vd_device_error(int* flags, int reset);

#ifdef __cplusplus
}
#endif
#endif /* VARDYN_GB300_H */
