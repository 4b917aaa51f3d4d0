/*
 * les_gb300.h -- C ABI of the GB300-native per-timestep spectral core of the
 * KhaledGhannam/LES large-eddy-simulation code.
 *
 * Every entry point replaces one Fortran external subroutine of the reference
 * (cited as file:line in the reference tree).  The Fortran arrays keep their
 * shape and column-major layout:
 *
 *   real field     double[nz][ny][ld]      ld = nx+2          (ld,ny,nz)
 *   complex plane  double[ny][lh][2]       lh = nx/2+1        (lh,ny) view
 *   padded field   double[nz][ny2][ld_big] ny2 = 3ny/2, ld_big = 3nx/2+2
 *   pressure       double[nz+1][ny][ld]    levels 0..nz-1 valid on exit
 *   surface plane  double[ny][nx]          (nx,ny)
 *
 * nz is the Fortran array extent (number of uvp levels + 1).  All pointers
 * passed to the per-routine entry points are HOST pointers unless the context
 * was switched to device-pointer mode with les_ctx_set_pointer_mode().
 *
 * Return value: 0 (LES_OK) or a negative les_status.  The reference prints a
 * message and calls `stop`; the Fortran shim turns a negative status into the
 * same message plus `stop`.
 *
 * Threading: one context per ensemble member; a context is bound to one CUDA
 * stream and is not thread-safe.  Different contexts may be driven from
 * different host threads.
 */
#ifndef LES_GB300_H
#define LES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum les_status {
  LES_OK = 0,
  LES_ERR_ARG = -1,         /* bad argument, shape or size                     */
  LES_ERR_CUDA = -2,        /* CUDA runtime error (message: les_last_error)    */
  LES_ERR_OOM = -3,         /* device allocation failed                        */
  LES_ERR_PIVOT = -4,       /* zero pivot: tridag_array.f90:34-37,62-67 `stop` */
  LES_ERR_CFL = -5,         /* CFLu > 0.1 or < 0: main.f90:455-458 `stop`      */
  LES_ERR_NAN = -6,         /* non-finite value detected in the state          */
  LES_ERR_TIMEOUT = -7,     /* bounded device wait expired                     */
  LES_ERR_STATE = -8,       /* call made before the required set-up            */
  LES_ERR_UNSUPPORTED = -9, /* size or mode not supported                      */
  LES_ERR_IO = -10          /* file open / read / write failed, bad record     */
} les_status;

/* Run configuration.  Mirrors the compile-time parameters of param.f90 and
 * the run-time namelist param_nml (param.f90:183-190), which the reference
 * fixes at compile time; here they are per-context run-time values. */
typedef struct les_config {
  int nx, ny, nz;       /* param.f90:56   grid; nz = uvp levels + 1             */
  int model;            /* param.f90:115  5 = Lagrangian scale-dependent,
                                          4 = Lagrangian scale-invariant,
                                          3 = plane-averaged scale-dependent,
                                          2 = standard dynamic (plane-averaged),
                                          7 = model 5 plus the Lagrangian
                                              scale-dependent SGS Prandtl number
                                              of the scalars (s_flag, precision 0 or 2) */
  int s_flag;           /* param.f90:158  1 = active potential temperature      */
  int initu;            /* param.f90:79   0 = Euler first momentum step         */
  int initsc;           /* param.f90:79   0 = Euler first scalar step           */
  int cs_count;         /* param.f90:100  steps between dynamic Cs updates (5)  */
  int jt_total0;        /* total_time.dat (param.f90:203-214) step offset        */
  int precision;        /* 0 = FP64 throughout, 1 = FP32-mixed form,
                                          2 = FP64 state and arithmetic with
                                              float-float (about 48-bit) transforms */
  int rmsdiv_every;     /* main.f90:451   rmsdiv/CFL diagnostic period (500)    */
  int q_flag;           /* main.f90:274   1 = humidity qmix (scalars_module_q.f90)
                                          advanced after theta; needs s_flag.
                                          0 = qmix identically zero (not stored) */
  double l_x, l_y;      /* param.f90:62   horizontal box (nondimensional)       */
  double lz_over_zi;    /* param.f90:63   L_z / z_i                             */
  double z_i;           /* param.f90:63   [m]                                   */
  double u_star;        /* param.f90:69   [m/s]                                 */
  double dt;            /* param.f90:219  nondimensional time step              */
  double vonk;          /* param.f90:98   von Karman constant                   */
  double t_scale;       /* param.f90:82   [K]                                   */
  double dtdz_top;      /* param.f90:81   [K/m]                                 */
  double pr;            /* param.f90:53   SGS Prandtl number                    */
  double g;             /* param.f90:177  [m/s^2]                               */
  double q_scale;       /* param.f90:85   humidity scale [g/kg]                 */
  double dqdz_top;      /* param.f90:83   humidity gradient at the lid [g/kg/m] */
} les_config;

/* State arrays that mirror the reference's module arrays (sim_param.f90:18-38,
 * sgsmodule.f90:8-34, scalars_module.f90:31-36, bottombc.f90:9-16). */
typedef enum les_field {
  LES_U = 0, LES_V, LES_W, LES_THETA,
  LES_DUDX, LES_DUDY, LES_DUDZ, LES_DVDX, LES_DVDY, LES_DVDZ,
  LES_DWDX, LES_DWDY, LES_DWDZ,
  LES_RHSX, LES_RHSY, LES_RHSZ, LES_RHSX_F, LES_RHSY_F, LES_RHSZ_F,
  LES_DPDX, LES_DPDY, LES_DPDZ,
  LES_TXX, LES_TXY, LES_TYY, LES_TXZ, LES_TYZ, LES_TZZ,
  LES_DIVTX, LES_DIVTY, LES_DIVTZ,
  LES_P,                 /* (ld,ny,0:nz) */
  LES_F_LM, LES_F_MM, LES_F_QN, LES_F_NN, LES_BETA, LES_CS_OPT2, LES_NU_T,
  LES_U_LAG, LES_V_LAG, LES_W_LAG,
  LES_RHS_T, LES_RHS_TF, LES_BETA_SCAL, LES_DTDX, LES_DTDY, LES_DTDZ,
  LES_S11, LES_S12, LES_S13, LES_S22, LES_S23, LES_S33,   /* calc_Sij output */
  /* humidity (scalars_module_q.f90:17-27; stored only when q_flag = 1) */
  LES_Q, LES_RHS_Q, LES_RHS_QF, LES_DQDX, LES_DQDY, LES_DQDZ,
  /* model 7 (sgsmodule.f90:8-34; stored only when model = 7): the scalar
   * Lagrangian averages, the turbulent Prandtl number, the scalar path's
   * Lagrangian velocity sums and the time scales lagrange_Sdep leaves */
  LES_G_LM, LES_G_MM, LES_G_QN, LES_G_NN, LES_PR_T,
  LES_U_LAG_S, LES_V_LAG_S, LES_W_LAG_S, LES_TN_LMMM, LES_TN_QNNN,
  /* surface planes (nx,ny) */
  LES_ZO, LES_WT_S, LES_USTAR_AVG, LES_PHI_M, LES_PSI_M, LES_PSI_M0,
  LES_PHI_H, LES_PSI_H, LES_PSI_H0, LES_SGS_T3_SFC,
  LES_WQ_S,              /* bottombc.f90:15 surface moisture flux [g/kg m/s] (q_flag) */
  LES_SGS_Q3_SFC,        /* scalars_module_q.f90:23 sgs_q3(:,:,1) (q_flag)          */
  LES_NUM_FIELDS
} les_field;

typedef struct les_ctx les_ctx;

/* ---- context ------------------------------------------------------------ */
/* Replaces init_fft / init_wavenumber (fft.f90:35-81) and the two
 * test_filter_init calls of main.f90:166-170; allocates the device mirrors of
 * the module arrays and all scratch.  Fields start at zero, as the reference's
 * static module storage does. */
int les_ctx_create(const les_config* cfg, les_ctx** out);
int les_ctx_destroy(les_ctx* ctx);
/* 0 = per-routine array arguments are host pointers (default), 1 = device
 * pointers, each 16-byte aligned (cudaMalloc'd arrays and whole-plane offsets
 * into them are); a misaligned one returns LES_ERR_ARG. */
int les_ctx_set_pointer_mode(les_ctx* ctx, int device_pointers);
/* Stream the context launches on (a cudaStream_t, passed as void*). */
void* les_ctx_stream(les_ctx* ctx);
/* Replace the context's stream by one of the given CUDA priority (lower is
 * more urgent; clamped to the device's range), after waiting for the work
 * queued on the old one.  A server gives members whose steps take longest
 * the most urgent streams so their steps are not starved by many small
 * ones.  No counterpart in the reference. */
int les_ctx_set_priority(les_ctx* ctx, int priority);
/* Bytes of device memory this context holds. */
size_t les_ctx_device_bytes(const les_ctx* ctx);
/* Estimated device bytes for a configuration (admission control). */
size_t les_estimate_device_bytes(const les_config* cfg);
const char* les_last_error(void);
/* Kernels launched by this library so far (all contexts, diagnostic). */
unsigned long long les_kernel_launch_count(void);

/* ---- state transfer ------------------------------------------------------ */
/* bottombc.f90:23-59 (patches): zo = roughness / z_i (nondimensional), wt_s =
 * kinematic surface heat flux [K m/s]; both (nx,ny). */
int les_set_surface(les_ctx* ctx, const double* zo, const double* wt_s);
/* Copy one module array host -> device / device -> host.  Real fields are
 * (ld,ny,nz), LES_P is (ld,ny,nz+1), surface planes are (nx,ny).  A
 * precision-1 context holds the horizontal velocity and theta gradients,
 * S_ij, Nu_t and tau_ij in FP32 (same layout, FP32 values in the first half of the
 * array); these copies and les_sync_* narrow / widen them, and
 * les_field_device_ptr returns that FP32 storage.  The per-routine entries
 * les_convec, les_sgs_stag, les_wallstress and les_theta_all_in_one need a
 * precision-0 or precision-2 context.  Precision 1 runs model 5. */
int les_set_field(les_ctx* ctx, les_field f, const double* host);
int les_get_field(les_ctx* ctx, les_field f, double* host);
/* Device address of a module array (for zero-copy use by the caller).  The
 * fused step takes RHSx_f = RHSx (and RHSy, RHSz, RHS_T) by exchanging the
 * two buffers, so those addresses alternate from step to step. */
double* les_field_device_ptr(les_ctx* ctx, les_field f);
size_t les_field_elems(const les_ctx* ctx, les_field f);
/* Bind Fortran module arrays once; les_sync_* then copy all bound arrays. */
int les_register_field(les_ctx* ctx, les_field f, double* host);
int les_sync_from_host(les_ctx* ctx);
int les_sync_to_host(les_ctx* ctx);
/* Step counters (param.f90:147-148). */
int les_get_counters(les_ctx* ctx, int* jt, int* jt_total);

/* Running statistics, io.f90:403-1218 (MM_XYZ_Out): time averages of 133
 * quantities on the (nx,ny,nz-1) grid (first to third moments of the
 * velocity, pressure, theta and qmix interpolated to the w nodes, fluxes,
 * gradients, SGS stresses and their products with strains and velocities,
 * pressure transport, the thermodynamic diagnostics), held on the device in
 * FP64.  les_stats_enable allocates them (133 nx ny (nz-1) doubles) and
 * zeroes them; with auto_accumulate = 1, les_step and les_step_graph
 * accumulate after every step whose jt is a multiple of c_count, as
 * output_loop does (io.f90:211-213; needs s_flag).  les_stats_accumulate is
 * one call of MM_XYZ_Out's accumulation on the current module state
 * (weight c_count / p_count; every statistic zeroed first when jt_total <=
 * c_count, io.f90:457-502).  The reference writes and zeroes two groups of
 * statistics every p_count and 2 p_count steps (io.f90:966-1217): the
 * caller reads them with les_stats_get and zeroes them with les_stats_reset
 * (group 1 or 2); les_stats_group tells each statistic's group (0: the
 * reference never zeroes it, atxy).  Statistic i (0 <= i < les_stats_count())
 * is named by les_stats_name(i) after the reference's array (au, u2, awt,
 * at11s11, azlcl_all, ...).  The output files themselves stay with the
 * caller.  Thermodynamic statistics use qmix = 0 without humidity, as the
 * reference does. */
int les_stats_enable(les_ctx* ctx, int c_count, int p_count, int auto_accumulate);
int les_stats_accumulate(les_ctx* ctx);
int les_stats_count(void);
const char* les_stats_name(int i);
int les_stats_group(int i);
int les_stats_get(les_ctx* ctx, int i, double* host);  /* (nx,ny,nz-1) */
int les_stats_reset(les_ctx* ctx, int group);

/* Whole-member state image, for a server that evicts a member from the
 * device and resumes it later: every module array in its device storage
 * (the FP32-held fields of a precision-1 context as they are) plus the step
 * counters, behind a header naming the configuration.  A context created
 * with the same configuration and surface and restored from the image
 * continues bit for bit as the saved one would have.  les_state_save fills a
 * host buffer of at least les_state_bytes bytes (pinned memory copies
 * fastest) and waits for the copies; les_state_restore refuses an image of
 * another configuration (LES_ERR_ARG).  No counterpart in the reference (its
 * restart record, les_checkpoint_write, keeps the arrays of io.f90:1314-1338
 * only, and a restart from it starts the Lagrangian sums and counters anew). */
size_t les_state_bytes(const les_ctx* ctx);
int les_state_save(les_ctx* ctx, void* host, size_t bytes);
int les_state_restore(les_ctx* ctx, const void* host, size_t bytes);

/* ---- checkpoint record ----------------------------------------------------- */
/* io.f90:1314-1338 `checkpoint` (written by output_final, io.f90:1347-1383,
 * and into output/vel_scNNNNNN.out, io.f90:223-233) and its reader
 * initial.f90:54-114 (with scalars) / :128-160 (without), model 5, not
 * inilag: one Fortran unformatted sequential record holding, with scalars,
 *   u, v, w, theta, qmix, RHSx, RHSy, RHSz, RHS_T, RHS_q   (ld,ny,1:nz) each,
 *   sgs_t3(:,:,1), sgs_q3(:,:,1)                          (ld,ny),
 *   psi_m, psi_m0, psi_h, psi_h0                          (nx,ny),
 *   Cs_opt2, F_LM, F_MM, F_QN, F_NN, G_LM, G_MM, G_QN, G_NN, Pr_t (ld,ny,nz);
 * without scalars u, v, w, RHSx, RHSy, RHSz, Cs_opt2, F_LM, F_MM, F_QN, F_NN.
 * Arrays this build does not carry are written as a model-5 run of the
 * reference holds them (G_* zero, Pr_t = Pr; qmix, RHS_q and sgs_q3 zero when
 * q_flag = 0, the context's arrays when q_flag = 1) and skipped on reading.  les_checkpoint_read takes only a record of exactly
 * its configuration's list (returning LES_ERR_IO, with no field changed,
 * for any other length).  The record keeps no step counters (the reference keeps
 * jt_total in total_time.dat): a restart creates its context with
 * jt_total0 = the steps taken, initu = 1 and initsc = 1, then reads the file.
 * Record format: gfortran / Intel Fortran unformatted sequential, 4-byte
 * little-endian markers around subrecords of at most 2147483639 bytes (a
 * negative leading marker: another subrecord follows; a negative trailing
 * marker: one precedes).  No counterpart in the reference for the functions
 * themselves (its Fortran runtime does this I/O). */
int les_checkpoint_write(les_ctx* ctx, const char* path);
int les_checkpoint_read(les_ctx* ctx, const char* path);
/* The record layer alone (host only, needs no context or GPU): write the
 * concatenation of nparts buffers as one record (append 0: new file;
 * max_subrecord <= 0: the standard 2147483639 bytes), or read the record at
 * byte offset into the buffers -- the record must hold at least their total;
 * the rest is skipped, as a Fortran read of a shorter list does -- returning
 * the record's length and the offset of the next record. */
int les_fortran_record_write(const char* path, int append, const void* const* parts, const size_t* nbytes,
                             int nparts, long long max_subrecord);
int les_fortran_record_read(const char* path, long long offset, void* const* parts, const size_t* nbytes,
                            int nparts, long long* record_bytes, long long* next_offset);

/* ---- fused time step ------------------------------------------------------ */
/* main.f90:202-478: nsteps iterations of the time loop on the device-resident
 * state (obukhov, filt_da, ddz, wallstress, sgs_stag, theta_all_in_one,
 * divstress, convec, AB2, press_stag_array, project, rmsdiv). */
int les_step(les_ctx* ctx, int nsteps);
/* Same as les_step, but every step (except the first, whose control flow is
 * special, and the rmsdiv/CFL diagnostic steps, which synchronise) is replayed
 * from a CUDA graph captured on first use; one graph per step variant
 * (dynamic-model step or not, Cs^2 override on or off).  No counterpart in the
 * reference (its time loop is main.f90:202-509). */
int les_step_graph(les_ctx* ctx, int nsteps);
/* Captures and instantiates the graphs les_step_graph will replay for the
 * next steps of both kinds (with and without the dynamic-model update) and
 * both RHS buffer parities, without running a step (counters and state are
 * unchanged), so a serving loop does not capture on its own path.  No
 * counterpart in the reference. */
int les_step_graph_prepare(les_ctx* ctx);
/* Times candidate launch shapes of the plane-transform kernels for this grid
 * size (kx columns per CTA of the y pass, rows per CTA of the x pass) and
 * keeps the fastest; results are cached per grid size for the process.
 * No counterpart in the reference. */
int les_autotune(les_ctx* ctx, int* tx64, int* tx32, int* rpc_scale);

/* ---- ensembles --------------------------------------------------------------
 * Independent members (any sizes) advanced together: one CUDA graph launch
 * per ensemble step runs one step of every member, each on its own stream
 * branch, so the members' work overlaps on the device.  Members must share
 * cs_count and the step counter.  No counterpart in the reference (nproc = 1
 * runs one member per process). */
typedef struct les_ensemble les_ensemble;
int les_ensemble_create(les_ctx* const* members, int n, les_ensemble** out);
int les_ensemble_step(les_ensemble* e, int nsteps);
void* les_ensemble_stream(les_ensemble* e);
int les_ensemble_destroy(les_ensemble* e);

/* rmsdiv.f90:1-113 on the start-of-step derivatives of the last step, and
 * timestep_conditions (scalars_module2.f90:22-70): cfl[0]=CFLu, cfl[1]=visc. */
int les_rmsdiv(les_ctx* ctx, double* rms);
int les_timestep_conditions(les_ctx* ctx, double* cflu, double* visc_stab);

/* ---- per-routine entry points (array arguments) --------------------------- */
/* ddx.f90:1-31 / ddy.f90:1-31 : spectral derivative of nlev planes. */
int les_ddx(les_ctx* ctx, double* dfdx, const double* f, int nlev);
int les_ddy(les_ctx* ctx, double* dfdy, const double* f, int nlev);
/* ddxy.f90:1-29 */
int les_ddxy(les_ctx* ctx, double* dfdx, double* dfdy, const double* f, int nlev);
/* filt_da.f90:3-42 : f <- Nyquist-filtered f, plus dfdx, dfdy. */
int les_filt_da(les_ctx* ctx, double* f, double* dfdx, double* dfdy, int nlev);
/* ddz_uv.f90:5-57, ddz_w.f90:6-51 (nz levels; untouched levels kept). */
int les_ddz_uv(les_ctx* ctx, double* dfdz, const double* f);
int les_ddz_w(les_ctx* ctx, double* dfdz, const double* f);
/* padd.f90:1-26 / unpadd.f90:1-22 on nplanes complex planes. */
int les_padd(les_ctx* ctx, double* u_big, const double* u, int nplanes);
int les_unpadd(les_ctx* ctx, double* cc, const double* cc_big, int nplanes);
/* dealias1.f90:1-31 / dealias2.f90:1-33 on nlev planes. */
int les_dealias1(les_ctx* ctx, const double* u, double* u_big, int nlev);
int les_dealias2(les_ctx* ctx, double* u, double* u_big, int nlev);
/* test_filtermodule.f90:13-30 : in-place filter of nplanes (ld,ny) planes
 * with transfer function G (lh,ny) that carries the 1/(nx*ny) normalisation. */
int les_test_filter(les_ctx* ctx, double* f, const double* G, int nplanes);
/* test_filtermodule.f90:32-63 : G for filter width alpha*delta. */
int les_test_filter_init(les_ctx* ctx, double alpha, double* G);
/* Plain unnormalised in-place 2-D real transforms of nplanes planes
 * (rfftwnd_f77_one_real_to_complex / complex_to_real with the plans of
 * fft.f90:40-47); big = 1 selects the 3/2-padded plan. */
int les_fft_r2c(les_ctx* ctx, double* planes, int nplanes, int big);
int les_fft_c2r(les_ctx* ctx, double* planes, int nplanes, int big);
/* Measurement (no counterpart in the reference): between les_profile_begin
 * and les_profile_end, every launch of one transform-kernel family on the
 * context's stream (eager steps, not graph replays) is bracketed by CUDA
 * events.  family: 1 FP64 y-pass, 2 FP32 y-pass, 3 FP64 x-pass, 4 FP32
 * x-pass; at most max_launches launches are measured.  end returns the
 * launches measured, their summed device time (ms) and summed algorithmic
 * bytes (each launch's inputs read once and outputs written once).  One
 * session per process at a time. */
/* Self-test (no counterpart in the reference): compares the library's
 * integer-pipe float<->double conversions with the hardware conversions on n
 * generated values (random bit patterns, the float range, halfway cases);
 * *mismatches receives the number of results whose bits differ. */
int les_selftest_conversions(size_t n, unsigned long long seed, unsigned long long* mismatches);
int les_profile_begin(les_ctx* ctx, int family, int max_launches);
int les_profile_end(les_ctx* ctx, int* launches, double* ms, double* bytes);
/* tridag_array.f90:1-109 : a,b,c (lh,ny,nz+1) real; r,u (lh,ny,nz+1) complex. */
int les_tridag_array(les_ctx* ctx, const double* a, const double* b, const double* c,
                     const double* r, double* u);
/* No counterpart in the reference.  les_tridag_array without any device
 * allocation, for callers that cannot call cudaMalloc or let a library do it
 * for them: applications whose device memory is all handed out by their own
 * pool or arena, and code that must not allocate mid-run.  It needs no
 * les_ctx (creating one allocates).  a, b, c (lh,ny,n) real and r, u
 * (lh,ny,n) complex are device pointers on the current device (r, u 16-byte
 * aligned); n = nz+1 in the reference's call.  The Thomas coefficients go to
 * a fixed scratch array compiled into the library, held on every GPU that
 * loads it until the process exits: lh*ny*n <= LES_NOALLOC_TRIDAG_MAX_ELEMS
 * (2^21, 16 MiB of doubles), larger sizes return LES_ERR_ARG.  The first call
 * on each device looks up that array's address.  All calls share the array:
 * calls that overlap on the GPU (other streams or host threads on the same
 * device) race; serialise them.  Runs on `stream` (a cudaStream_t, 0 for the
 * default stream) and synchronises that stream on every call (twice: after
 * the row-1 pivot check and after the solve) to report a zero pivot as
 * LES_ERR_PIVOT, so it cannot be called inside stream capture or a CUDA
 * graph.  A zero b in row 1 returns LES_ERR_PIVOT before the solve runs and
 * leaves u as passed; modes the solve skips (kx = lh-1, ky = ny/2, and the
 * (0,0) mode beyond row 1) keep the caller's values beyond row 1, as
 * tridag_array.f90 leaves them. */
#define LES_NOALLOC_TRIDAG_MAX_ELEMS (1u << 21)
int les_tridag_array_noalloc(const double* a, const double* b, const double* c, const double* r,
                             double* u, int lh, int ny, int n, void* stream);
/* Routines that read the module arrays bound to the context. */
/* convec.f90:1-248 -> cx, cy, cz (ld,ny,nz), valid 1:nz-1. */
int les_convec(les_ctx* ctx, double* cx, double* cy, double* cz);
/* divstress_uv.f90:1-63 / divstress_w.f90:4-86 */
int les_divstress_uv(les_ctx* ctx, double* divt, const double* tx, const double* ty,
                     const double* tz);
int les_divstress_w(les_ctx* ctx, double* divt, const double* tx, const double* ty,
                    const double* tz);
/* press_stag_array.f90:1-294 on the context's u,v,w (u*) and divtz:
 * p_hat (ld,ny,0:nz) physical pressure, dfdx/dfdy (ld,ny,nz). */
int les_press_stag_array(les_ctx* ctx, double* p_hat, double* dfdx, double* dfdy);
/* sgs_stag.f90:3-364 on the context state (includes calc_Sij, the Lagrangian
 * accumulation, the dynamic-model dispatch and the tau_ij assembly). */
int les_sgs_stag(les_ctx* ctx);
/* lagrange_Sdep.f90:4-478 (calls interpolag_Sdep) with S_ij (ld,ny,nz). */
int les_lagrange_sdep(les_ctx* ctx, const double* S11, const double* S12, const double* S13,
                      const double* S22, const double* S23, const double* S33);
/* interpolag_Sdep.f90:2-380 on the context's F_* and u/v/w_lag. */
int les_interpolag_sdep(les_ctx* ctx);
/* lagrange_Ssim.f90:5-335 (model 4, calls interpolag_Ssim) with S_ij
 * (ld,ny,nz); interpolag_Ssim.f90:3-316 on the context's F_LM, F_MM and
 * u/v/w_lag. */
int les_lagrange_ssim(les_ctx* ctx, const double* S11, const double* S12, const double* S13,
                      const double* S22, const double* S23, const double* S33);
int les_interpolag_ssim(les_ctx* ctx);
/* scaledep_dynamic.f90:4-255 -> cs_opt2 (nz) with S_ij (ld,ny,nz). */
int les_scaledep_dynamic(les_ctx* ctx, double* cs_opt2, const double* S11, const double* S12,
                         const double* S13, const double* S22, const double* S23,
                         const double* S33);
/* std_dynamic.f90:1-136 (model 2) -> cs_opt2 (nz) with S_ij (ld,ny,nz) and
 * the context's u, v, w. */
int les_std_dynamic(les_ctx* ctx, double* cs_opt2, const double* S11, const double* S12, const double* S13,
                    const double* S22, const double* S23, const double* S33);
/* Model 7 (sgs_stag.f90:147-152): lagrange_scalar_Sdep.f90:1-467 computes
 * Cs2_Pr = Cs^2/Pr_t with Lagrangian averaging of the scalar's
 * L.M and Q.N along the pathlines (G_LM, G_MM, G_QN, G_NN, relaxed with the
 * time scales of lagrange_Sdep), re-filters theta (filt_da) and sets
 * Pr_t = Cs_opt2 / Cs2_Pr, Beta to the scalar's scale-dependence factor;
 * interpolag_scalar_Sdep.f90 moves G_* along the back-trajectories of
 * u_lag_s, v_lag_s, w_lag_s and resets them.  The scalars' SGS fluxes then
 * use Pr_t instead of Pr (scalars_module.f90:77-82).  Both act on the
 * module state of a model-7 context; cs2_pr is (ld,ny,nz). */
int les_lagrange_scalar_sdep(les_ctx* ctx, double* cs2_pr, const double* S11, const double* S12,
                             const double* S13, const double* S22, const double* S23, const double* S33);
int les_interpolag_scalar_sdep(les_ctx* ctx);
/* wallstress.f90:5-69, scalars_module.f90:508-690 (obukhov),
 * forcing.f90:128-219 (project), scalars_module.f90:57-171 (theta_all_in_one). */
int les_wallstress(les_ctx* ctx);
int les_obukhov(les_ctx* ctx);
int les_project(les_ctx* ctx);
int les_theta_all_in_one(les_ctx* ctx);
/* scalars_module_q.f90:31-141 q_all_in_one (filt_da and ddz_uv of qmix, the
 * lid gradient dqdz_top, scalar_q_RHS_calc :145-367, step_scalar_q :370-397)
 * on the context's module state; needs q_flag = 1 (else LES_ERR_STATE) and a
 * precision-0 or precision-2 context.  In les_step it runs after theta_all_in_one
 * (main.f90:273-274); qmix also enters calcbeta's virtual temperature
 * (scalars_module.f90:200-223) and obukhov's buoyancy flux
 * (scalars_module.f90:547-550). */
int les_q_all_in_one(les_ctx* ctx);
/* atm_thermodynamics.f90:25-60 thermo(): the diagnostic arrays of the module
 * from the context's theta and qmix, levels 1..nz-1, columns 1..nx (each
 * array (ld,ny,nz); padding columns and level nz are zero): actual and
 * virtual temperature [nondimensional, T_scale], saturation vapour pressure
 * [Pa], pressure [Pa], vapour pressure [Pa], saturation mixing ratio,
 * relative humidity from pressures and from mixing ratios, and the lifting
 * condensation level [m].  Nothing in the step reads them (main.f90:275);
 * the reference's periodic zlcl_parcel output files are not written.
 * Needs q_flag = 1 and s_flag = 1. */
int les_atm_thermodynamics(les_ctx* ctx, double* actual_T, double* actual_Tv, double* sat_vapor_pr,
                           double* pr_atm, double* vapor_pr, double* sat_qmix, double* rel_hum,
                           double* rel_hum_q, double* zlcl_all);

#ifdef __cplusplus
}
#endif

#endif /* LES_GB300_H */
