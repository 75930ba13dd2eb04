/*
 * suli_gpu.h -- C ABI of the GB300 (sm_103a) implementation of SuLi-IC's
 * per-time-step hot path.
 *
 * SuLi's hot routines are argument-less Fortran subroutines that talk through
 * module globals (SuLi-IC/0_modules.f90:2-325) and are called from the time
 * loop in SuLi-IC/1_principal.f90:69-124.  This header replaces each of them
 * with one entry point that acts on a device-resident case held by a handle.
 * A Fortran shim (ISO_C_BINDING interfaces over these entry points) keeps the
 * original subroutine names so the time loop is unchanged.
 *
 * Conventions
 *   - Every entry point returns an int status: 0 = SULI_OK, >0 an error or
 *     warning code (below).  suli_last_error() gives the text of the last one.
 *   - Host arrays crossing the boundary use the reference's own layout:
 *     Fortran column-major, i (x) fastest, with the reference's lower bounds
 *     (e.g. u is (0:nx+2, 0:ny+1, 0:nz+1)); suli_field_shape() reports the
 *     bounds of every field id.
 *   - Ownership: after suli_upload_field() the device owns the data; host
 *     arrays are only read/written during the call.
 *   - Threading: one host thread per handle; not re-entrant.
 *   - There is no CPU fallback: a handle cannot be created without a CUDA
 *     device and a missing device is reported as SULI_NO_DEVICE.
 */
#ifndef SULI_GPU_H
#define SULI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SULI_OK              0
#define SULI_CG_MAXITER      1  /* warning: "pulou pressao", 9_grad.f90:590 */
#define SULI_VOL_LOOP_CAP    2  /* volume-correction loop capped, 14_level_set.f90:243 */
#define SULI_DEVICE_TIMEOUT  3  /* a bounded device wait for a TMA copy (the staged convdiff)
                                   gave up after one second; the step's results for that case
                                   are not valid (checked where SULI_NONFINITE is and at the
                                   end of suli_step) */
#define SULI_BAD_CONFIG      4  /* replaces the reference's STOPs */
#define SULI_BAD_ARG         5
#define SULI_CUDA_ERROR      6
#define SULI_NO_DEVICE       7
#define SULI_OUT_OF_MEMORY   8
#define SULI_CG_STALLED      9  /* warning (mixed form, no counterpart in the reference): the FP64
                                   residual of the pressure refinement stopped falling before the
                                   tolerance; the solve ends on its last pass */
#define SULI_NONFINITE      10  /* a case's state holds NaN or Inf: its volume integral or its
                                   max|div| is not finite (checked by suli_level_set, i.e. once per
                                   step of suli_step, and by suli_conmassa); the reference has no
                                   such check and runs on with the NaNs */

/* ---- precision of a case ----------------------------------------------- */
#define SULI_PREC_FP64   0  /* plain form: FP64 storage and arithmetic */
#define SULI_PREC_MIXED  1  /* FP32 storage/stencils, FP64 refinement + sums */

/* ---- CG stopping rule --------------------------------------------------- */
#define SULI_CG_TOL_ABS  0  /* reference rule: r.r > cg_tol/(nx*ny*nz), 9_grad.f90:393 */
#define SULI_CG_TOL_REL  1  /* norm(r) > cg_tol norm(b), scaled system, b = q / sqrt(D) */

/*
 * suli_params mirrors the module variables the hot path reads
 * (0_modules.f90 disc/cond/param/les/ls_param, read by parametros()
 * 2_iniciais.f90:11-123).  The trailing block holds the build's own
 * knobs, each defaulting to the reference behaviour when zero-filled
 * through suli_default_params().
 */
typedef struct suli_params {
    int32_t nx, ny, nz;            /* cells */
    double  dx, dy, dz;            /* m */
    double  dt;                    /* dt0, s */
    int32_t t_tempo;               /* 0 Euler, 1 RK2, 2 RK3, 3 AB2, 4 AB3 */
    int32_t der;                   /* 3 = 2nd-order upwind (only one supported) */
    int32_t adv_type;              /* 1 = classical advective form */
    int32_t ibm_t;                 /* 0 none, 2 image-point IBM */
    int32_t obst_t;                /* 0 none, nonzero: obstacle fields uploaded */
    int32_t m_turb;                /* 0 none, 1 Smagorinsky, 2 k-equation LES, 3 k-equation DES
                                      (5_viscosidade.f90:74-145) */
    int32_t t_press;               /* 1 projection, 2 implicit pressure algorithm (IPA: exp_press,
                                      11_diversos.f90:455-495; graddin after the RK loop with the
                                      density rho_f1, 9_grad.f90:103-115; 1_principal.f90:82,111) */
    int32_t mms_t;                 /* 0 none, 1 steady MMS source */
    int32_t ccx0, ccxf, ccy0, ccyf, ccz0, cczf;  /* 0 periodic,1 free-slip,2 no-slip,3 prescribed,4 outflow(xf) */
    double  gx, gz;                /* gravity components (reference: 9.80665*sin/cos(atan(decliv))) */
    double  csmag;                 /* Smagorinsky constant */
    double  alpha1;                /* interface half-width in cells */
    double  rho_f1, mu_f1;         /* fluid where ls < 0 (air) */
    double  rho_f2, mu_f2;         /* fluid where ls > 0 (water) */
    double  uinicial, iturb;       /* inflow speed and perturbation for ccx0 = 3 */
    int32_t omp_t;                 /* reference CG reduction mode; no effect on the GPU */
    /* ---- build-specific knobs ---- */
    int32_t reinit_max_iter;       /* reference: 3 (14_level_set.f90:389) */
    int32_t cg_max_iter;           /* reference: 10000 (9_grad.f90:398) */
    int32_t cg_tol_mode;           /* SULI_CG_TOL_ABS (reference) or SULI_CG_TOL_REL */
    double  cg_tol;                /* reference: 1e-4 with SULI_CG_TOL_ABS */
    int32_t precision;             /* SULI_PREC_FP64 or SULI_PREC_MIXED */
    int32_t project_under_mms;     /* 1: run graddin/posdin/contorno(1) even when mms_t>0 */
    int32_t vol_loop_max;          /* cap of the volume-correction loop (reference: none) */
    int32_t mixed_precond;         /* mixed form: FP32 passes as 0 Jacobi-scaled CG (graddin's own
                                      iteration), 1 CG preconditioned by a multigrid V-cycle */
    uint64_t seed;                 /* counter-based RNG seed for the inflow perturbation */
    int32_t t_tens;                /* 0 none, 1 surface tension (2_iniciais.f90:56; 14_level_set.f90:519-567,
                                      :660-704; 11_diversos.f90:383-395) */
    double  sigma;                 /* surface tension coefficient, N/m (reference: 0.0728) */
    double  cmu, cdes;             /* k-equation constants: nut = cmu sqrt(ka) delta; DES limiter
                                      constant (2_iniciais.f90:79-80) */
    double  lcar;                  /* k-equation dissipation length: the reference's max(prof, ampl)
                                      (5_viscosidade.f90:94) */
    int32_t esp_type;              /* sponge layer over the last 1 m in x: 0 none, 1 graded with the
                                      depth, 2 linear (3_contorno.f90:1011-1103) */
    int32_t wave_t;                /* inflow waves for ccx0 = 3: 0 none, 1 Stokes I, 2 Stokes II,
                                      5 Stokes V (boundary_waves, 3_contorno.f90:1189-1319) */
    double  a_w, f_w, n_w, h0_f;   /* wave amplitude, angular frequency, wave number, still depth:
                                      waves_coef's results (3_contorno.f90:1323-1445, run by the
                                      host's iniciais, 2_iniciais.f90:241-245) */
    double  aeta[5], avel[5];      /* Stokes V surface and velocity coefficients (waves_coef) */
    int32_t outflow_flux;          /* with ccxf = 4 (free outflow), 1: contorno(2) adds one uniform
                                      correction to the outflow faces u(nx+1, 1:ny, 1:nz) so that their
                                      flux equals the inflow faces' u(1, 1:ny, 1:nz) (no counterpart in
                                      the reference, whose free outflow leaves a net boundary flux that
                                      the all-Neumann pressure equation of graddin cannot absorb);
                                      0: the reference's free outflow */
    int32_t dz_t;                  /* z spacing: 0 uniform dz (SuLi-IC); 1 the variable spacing of
                                      SuLi-ICdz, dz(k) = dzmin + (dzmax - dzmin) k / nz for k = 0..nz+1
                                      (dz_dist, SuLi-ICdz/2_iniciais.f90:326-406), with the ICdz
                                      stencils (weighted z interpolations, dz(k)/dzz(k) in the z
                                      differences, graddin/posdin/CONMASSA, the WENO z lines);
                                      supported for the plain two-fluid flow (m_turb = 0, no IBM,
                                      surface tension, IPA, MMS, sponge, waves or inflow) */
    double  dzmin, dzmax;          /* dz_t = 1: the spacing at k = 0 and at k = nz (dz is ignored;
                                      max(dx, dy, dzmin) is the level set's dx1, as upstream) */
} suli_params;

/* ---- field ids (reference module arrays) -------------------------------- */
enum suli_field {
    SULI_F_U = 0,    /* u   (0:nx1+1, 0:ny+1, 0:nz+1)  velpre */
    SULI_F_V,        /* v   (0:nx+1, 0:ny1+1, 0:nz+1) */
    SULI_F_W,        /* w   (0:nx+1, 0:ny+1, 0:nz1+1) */
    SULI_F_PRD1,     /* prd1 (0:nx+1, 0:ny+1, 0:nz+1) */
    SULI_F_PRD,      /* prd  (0:nx+1, 0:ny+1, 0:nz+1) */
    SULI_F_LS,       /* ls   (nx, ny, nz)  ls_param */
    SULI_F_HS,       /* hs   (nx, ny, nz) */
    SULI_F_RHO,      /* rho  (nx, ny, nz) */
    SULI_F_LS_MU,    /* ls_mu (nx, ny, nz) */
    SULI_F_MU,       /* mu   (nx, ny, nz)  les */
    SULI_F_MUT,      /* mut  (nx, ny, nz) */
    SULI_F_XMU,      /* xmu  (nx1, ny, nz) */
    SULI_F_YMU,      /* ymu  (nx, ny1, nz) */
    SULI_F_ZMU,      /* zmu  (nx, ny, nz1) */
    SULI_F_FU,       /* Fu   (nx1, ny, nz)  vartempo */
    SULI_F_FV,       /* Fv   (nx, ny1, nz) */
    SULI_F_FW,       /* Fw   (nx, ny, nz1) */
    SULI_F_U0, SULI_F_V0, SULI_F_W0,
    SULI_F_FU0, SULI_F_FV0, SULI_F_FW0,
    SULI_F_FU1, SULI_F_FV1, SULI_F_FW1,
    SULI_F_DIV,      /* div  (nx, ny, nz) */
    SULI_F_TF_U, SULI_F_TF_V, SULI_F_TF_W,   /* MMS sources, mms_m */
    SULI_F_OBS_LSX,  /* obs_lsx (nx1, ny, nz)  obst */
    SULI_F_OBS_LSY,  /* obs_lsy (nx, ny1, nz) */
    SULI_F_OBS_LSZ,  /* obs_lsz (nx, ny, nz1) */
    SULI_F_OBS_LSS,  /* obs_lss (nx, ny, nz) */
    SULI_F_ID_IBMX,  /* id_ibmx (nx1, ny, nz), int32 */
    SULI_F_ID_IBMY,
    SULI_F_ID_IBMZ,
    SULI_F_ID_IBM,   /* id_ibm (nx, ny, nz), int32 */
    SULI_F_BXX0,     /* bxx0 (0:ny+1, 0:nz+1) inflow u at i = 0 */
    SULI_F_BXX1,     /* bxx1 (0:ny+1, 0:nz+1) inflow u at i = 1 */
    SULI_F_BLX1,     /* blx1 (ny, nz) inflow ls at i = 1 */
    SULI_F_OBS_LS,   /* obs_ls (nx1, ny1, nz1) obstacle level set at the cell corners, written by
                        obstaculo() for the field output (3_contorno.f90:905-911, 4_plot.f90:570) */
    SULI_F_HSX,      /* hsx (nx, ny, nz) surface-tension weight, heaviside (14_level_set.f90:563-567) */
    SULI_F_HSY,
    SULI_F_HSZ,
    SULI_F_KURV,     /* kurv (nx, ny, nz) interface curvature, curv_ls1 (14_level_set.f90:660-704) */
    SULI_F_KA,       /* ka (0:nx+1, 0:ny+1, 0:nz+1) turbulent kinetic energy, les; stored for
                        m_turb >= 2 only ("field not stored" otherwise, where the reference's ka is 0) */
    SULI_F_NUT,      /* nut (nx, ny, nz) modelled kinematic viscosity; stored for m_turb >= 2 */
    SULI_F_PRD0,     /* prd0 (0:nx+1, 0:ny+1, 0:nz+1) accumulated pressure of the IPA; t_press = 2 */
    SULI_F_PX,       /* px (nx1, ny, nz) explicit pressure force of the IPA (exp_press); t_press = 2 */
    SULI_F_PY,       /* py (nx, ny1, nz) */
    SULI_F_PZ,       /* pz (nx, ny, nz1) */
    SULI_F_BXZ0,     /* bxz0 (0:ny+1, 0:nz+1) inflow w at i = 0 (ccx0 = 3; the waves set it) */
    SULI_F_COUNT
};

/* ---- scalar ids ---------------------------------------------------------- */
enum suli_scalar {
    SULI_S_T = 0,      /* simulated time t */
    SULI_S_DT,         /* current (stage) dt */
    SULI_S_VOL_INI,
    SULI_S_VOL_INS,
    SULI_S_MAXDIV,     /* maxval(abs(div)) of the last suli_conmassa */
    SULI_S_IT,         /* time-step counter (as double) */
    SULI_S_TT,         /* RK stage (as double) */
    SULI_S_RNG,        /* inflow perturbation draws so far (calls of the ccx0 = 3 fill) */
    SULI_S_COUNT
};

typedef struct suli_diag {
    double  vol_ini, vol_ins, maxdiv, t;
    double  cg_res[3];          /* final CG r.r (scaled system) per RK stage */
    int32_t cg_iters[3];        /* CG iterations per RK stage of the last step */
    int32_t cg_outer[3];        /* mixed form: FP64 refinement passes per stage */
    int32_t reinit_iters;       /* reinit iterations (il) of the last level_set */
    int32_t vol_loops;          /* volume-correction passes of the last level_set */
    int32_t it;
    int32_t status_flags;       /* OR of warnings seen since the last read */
} suli_diag;

typedef struct suli_handle suli_handle;

/* Zero-fill + reference defaults (reinit 3, cg 10000, abs tol 1e-4, FP64). */
void suli_default_params(suli_params *p);

/* Extents of field f for params p, as Fortran lower/upper bounds. */
int suli_field_shape(const suli_params *p, int field, int lo[3], int hi[3]);

/* Replaces parametros()/init_variables1..7 (2_iniciais.f90:11-123,
 * 0_modules.f90:121-347): validates p and allocates one device case. */
int suli_create(const suli_params *p, suli_handle **out);
/* A batch of independent cases advanced in lockstep by the same launches
 * (uneven grids allowed; the scheme flags and precision must match). */
int suli_create_batch(const suli_params *p, int ncases, suli_handle **out);
int suli_num_cases(const suli_handle *h, int *ncases);
int suli_destroy(suli_handle *h);

/* Host <-> device copies of one field of case icase in the reference layout.
 * int32 for id_ibm*, double otherwise (the mixed form converts). */
int suli_upload_field(suli_handle *h, int icase, int field, const void *host);
int suli_download_field(suli_handle *h, int icase, int field, void *host);
/* The same copies for n (case, field, buffer) triples in one call: all are
 * queued on the handle's stream and the call synchronises once, at its end
 * (the per-field calls synchronise each).  The buffers must stay valid until
 * the call returns.  For a host that moves a batch's state every step (the
 * reference keeps everything in host memory, so it has no counterpart).
 * Page-locked host buffers (cudaHostAlloc, cudaHostRegister) are the fast
 * form: the mixed form's conversion kernel then reads or writes them in
 * place (no staging copy) and one launch covers every field of the list;
 * pageable buffers go through a device staging buffer one field at a time.
 * Both give the same bits. */
int suli_upload_fields(suli_handle *h, int n, const int32_t *cases, const int32_t *fields,
                       const void *const *host);
int suli_download_fields(suli_handle *h, int n, const int32_t *cases, const int32_t *fields, void *const *host);
int suli_set_scalar(suli_handle *h, int icase, int scalar, double value);
int suli_get_scalar(suli_handle *h, int icase, int scalar, double *value);

/* Parity runs: replay the CG iteration count of each RK stage and the
 * reinitialisation count of a reference run (-1 = free running). */
int suli_set_replay(suli_handle *h, const int32_t cg_iters[3], int32_t reinit_iters);

/* heaviside() 14_level_set.f90:508-594 plus the vol_ini sum of
 * level_set_ini() :187-194; call once after uploading ls. */
int suli_heaviside_init(suli_handle *h);

/* obstaculo() tail for ibm_t = 2 (3_contorno.f90:991-1002): after the
 * obstacle level sets obs_lsx/y/z/s are uploaded, reinitialise them and
 * build the integer image-point masks id_ibm* (ibm_posicoes, 15_ibm.f90:9-131). */
int suli_ibm_setup(suli_handle *h);

/* One entry point per reference subroutine. */
int suli_level_set(suli_handle *h);              /* 14_level_set.f90:204-273 */
int suli_contorno(suli_handle *h, int nlock);    /* 3_contorno.f90:11-662 */
int suli_visco(suli_handle *h);                  /* 5_viscosidade.f90:11-157 */
int suli_convdiff(suli_handle *h);               /* 6_convdiff.f90:14-167 */
int suli_complementos(suli_handle *h);           /* 11_diversos.f90:355-450 */
int suli_tempo(suli_handle *h);                  /* 11_diversos.f90:10-296 (uses stage tt, dt) */
int suli_graddin(suli_handle *h, int32_t *iters_out); /* 9_grad.f90:10-663 */
int suli_posdin(suli_handle *h);                 /* 10_pos.f90:1-99 */
/* exp_press (11_diversos.f90:455-495), t_press = 2 only: prd0 += prd1 and the
 * explicit pressure force px/py/pz from prd0 + prd1 over the face density,
 * which tempo adds to Fu/Fv/Fw (11_diversos.f90:21-45).  The IPA step calls it
 * before visco and graddin once after the RK loop, without posdin
 * (1_principal.f90:82,111).  SULI_BAD_CONFIG for t_press != 2. */
int suli_exp_press(suli_handle *h);
/* contorno_les (3_contorno.f90:666-790): the ghost values of ka, for the
 * cases with m_turb >= 2 (the k-equation loop of visco calls it on every
 * sub-stage; iniciais calls it once after setting ka, 2_iniciais.f90:216-235). */
int suli_contorno_les(suli_handle *h);
/* boundary_waves (3_contorno.f90:1189-1319), wave_t > 0: the inflow planes
 * bxx0, bxx1, bxz0 and ls(1, :, :) of the wave at the current time t; the
 * step calls it after tempo in every RK stage (1_principal.f90:93). */
int suli_boundary_waves(suli_handle *h);
int suli_conmassa(suli_handle *h, double *maxdiv_out); /* 4_plot.f90:386-394 */
int suli_mms_error(suli_handle *h, double err_out[4]); /* 13_mms.f90:391-451 */
/* Sets tt (1..ntt) and dt = a_dt(tt), as the RK loop of 1_principal.f90:86-87. */
int suli_set_stage(suli_handle *h, int tt);

/* The whole time step of 1_principal.f90:69-124 (without PLOT output),
 * nsteps times; captured once into a CUDA graph and replayed. */
int suli_step(suli_handle *h, int nsteps);

int suli_diagnostics(suli_handle *h, int icase, suli_diag *out);
int suli_synchronize(suli_handle *h);

/* Measurement support.  suli_get_stream: the CUDA stream (cudaStream_t)
 * every kernel of the handle is launched on, for events recorded by the
 * caller.  suli_profile(h, 1) starts counting kernel launches and timing the
 * CG iteration loop with CUDA events on that stream; suli_profile_read
 * returns the totals since then. */
typedef struct suli_profile_t {
    uint64_t launches;          /* kernels launched by the handle */
    double   cg_ms;             /* event time spent in CG iteration chunks */
    double   cg_cell_iters;     /* sum over cases of cells x CG iterations */
    double   cg_bytes_per_cell_iter; /* bytes the iteration kernels move per cell */
} suli_profile_t;
int suli_get_stream(suli_handle *h, void **stream);
int suli_profile(suli_handle *h, int enable);
int suli_profile_read(suli_handle *h, suli_profile_t *out);
/* Measurement only (no counterpart in the reference): time one kernel alone
 * over every case of the handle, `reps` launches between CUDA events on the
 * handle's stream.  kernel 0: the CG matrix-vector product (k_cgi_A),
 * 1: one red half-sweep of the multigrid smoother on the case grid (mixed form
 * with mixed_precond = 1 only), 2: the CG direction update (k_cgi_C),
 * 3: one whole one-pass red-black sweep of the smoother on the case grid
 * (mixed form with mixed_precond = 1 only).
 * Returns the mean time per launch and the algorithmic bytes one launch
 * moves.  The solver work arrays it touches are rebuilt by the next
 * suli_graddin. */
int suli_time_kernel(suli_handle *h, int kernel, int reps, double *ms_per_launch, double *bytes_per_launch);
/* Autotuner (no counterpart in the reference).  Launch shapes of the hot
 * kernels -- the planes per unit of the TMA-staged convdiff (8, 16, 32), the
 * largest multigrid level handled by the one-block coarse end of the V-cycle,
 * the blocks per SM of the one-pass multigrid smoother sweep -- are timed with
 * CUDA events on the handle's stream and the fastest kept; every choice gives
 * the same bits (only the partition of the work changes).  suli_step tunes a
 * handle once, after its first time step (the operator and the work arrays
 * exist by then; tuning touches only scratch arrays), unless the environment
 * sets SULI_TUNE=0; the choice is cached per device and workload shape
 * (precision, cases, cells, multigrid levels), so further handles of the same
 * shape reuse it.  suli_autotune tunes now (or applies the cached choice);
 * suli_get_tuning reports the current one. */
typedef struct suli_tuning {
    int32_t convdiff_planes;      /* planes per unit of the TMA-staged convdiff (0: gather kernel) */
    int32_t mg_block_cells;       /* largest level (cells) of the one-block V-cycle end; 0: none */
    int32_t sweep_blocks_per_sm;  /* blocks per SM of the multigrid sweep; 0: occupancy limit */
    int32_t tuned;                /* 1: chosen by timing (this handle or the cache), 0: defaults */
    double  default_ms;           /* the timed kernels at the defaults (one convdiff, one V-cycle, one sweep) */
    double  tuned_ms;             /* the same at the chosen shapes */
} suli_tuning;
int suli_autotune(suli_handle *h, suli_tuning *out);
int suli_get_tuning(suli_handle *h, suli_tuning *out);

/* PRTSCR (4_plot.f90:501-635), the field record of one case: written to
 * `path` as one Fortran unformatted sequential record (gfortran framing: a
 * 4-byte little-endian byte count before and after) of float32 arrays in
 * Fortran order -- x, y, z of the cell corners (nx+1, ny+1, nz+1), u, v, w
 * averaged to the corners, ls (nx, ny, nz), obs_ls at the corners (zero
 * without an obstacle), and with t_plot = 1 the pressure minus its value at
 * cell (nx, 1, nz) (prd0 + prd1 under the IPA), the three vorticity
 * components, nut and ka (zeros for m_turb < 2, as in the reference).  The record is formed on
 * the device and copied once into pinned host memory.  The file name and the
 * output cadence (dt_frame) are the caller's, as is the XDMF index (visu,
 * 12_paraview_3D.f90).  SULI_BAD_ARG when the file cannot be written or the
 * record exceeds 2^31 - 1 bytes. */
int suli_write_fields(suli_handle *h, int icase, const char *path, int t_plot);
/* restart_salva / restart_ini (11_diversos.f90:500-599, called from
 * 1_principal.f90:38 and :120-122) as a binary file: every field of every
 * case in the reference layouts (FP64; the IBM masks int32), t, it, dt, the
 * inflow draws and the stage, and per case vol_ini / vol_ins.  Unlike the
 * reference, which reads its text dump back and then resets t and it to
 * zero, suli_restart_load restores them, so a run that is saved, loaded into
 * a handle created with the same parameters and continued matches the run
 * that was never interrupted.  SULI_BAD_CONFIG when the file is not a
 * restart of this library or was written for other cases. */
int suli_restart_save(suli_handle *h, const char *path);
int suli_restart_load(suli_handle *h, const char *path);

/* Divergence and max|div| of a velocity field held in caller-owned device
 * memory: the reference CONMASSA divergence in FP64 (what suli_conmassa gives
 * for an FP64 handle; a mixed handle stores its div in FP32), allocating no
 * device memory (no counterpart in the reference: it exists for callers that
 * own every device buffer through their own allocator or memory budget, e.g.
 * a Fortran host whose arrays live in CUDA Fortran / OpenACC data regions).
 * u, v, w, div are device arrays in the reference layout: u(0:nx+2,0:ny+1,
 * 0:nz+1), v(0:nx+1,0:ny+2,0:nz+1), w(0:nx+1,0:ny+1,0:nz+2), div(1:nx,1:ny,
 * 1:nz), column-major; maxdiv is one device double.  Limit: nz <= 4096 (the
 * z-planes its built-in 32 KiB scratch holds); larger nz returns
 * SULI_BAD_ARG.  The scratch is one static device array shared by every
 * call: calls that overlap on the GPU race and must be serialised.  The first
 * call on each device looks up the scratch address; make it before any
 * stream capture.  Enqueued on `stream` (a cudaStream_t; NULL = default). */
int suli_conmassa_noalloc(const double *u, const double *v, const double *w, int32_t nx, int32_t ny,
                          int32_t nz, double dx, double dy, double dz, double *div, double *maxdiv,
                          void *stream);

/* Text of the last error on this thread (empty if none). */
int suli_last_error(char *buf, size_t len);

/* Device/runtime info for reports: SM count, clock, name. */
int suli_device_info(int *sm_count, char *name, size_t name_len);

#ifdef __cplusplus
}
#endif

#endif /* SULI_GPU_H */
