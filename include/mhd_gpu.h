/*
 * mhd_gpu.h -- C-ABI of libmhdgpu.so, the GB300 (sm_103a) implementation of
 * the cylindrical (r, phi, z) GLM-MHD TVD Runge-Kutta step of
 * github-nakasho/171026-1-3dhlld-cyli-gal.
 *
 * The reference is one C program whose step loop (main.c:316-393) calls three
 * functions on global arrays:
 *
 *     Setdt();          setdt.h:24       -> mhd_setdt()
 *     SpiralGravity();  spiralgravity.h:20 -> mhd_spiral_gravity()
 *     TVDRK();          tvdrungekutta.h:16 -> mhd_tvdrk()
 *
 * and stops the program on a bad dt (main.c:331-334) -> mhd_step() returns
 * MHD_ERR_DT instead.  A reference host keeps its globals, array layout
 * ([m][i][j][k], k fastest, FP64, one ghost cell per side) and file formats;
 * it hands its arrays to mhd_create()/mhd_upload() once and calls the step
 * functions in place of its own.
 *
 * Conventions: every function returns 0 (MHD_OK) or a negative MHD_ERR_*
 * code; nothing prints or exits.  A context is used by one host thread at a
 * time and owns one CUDA stream.  The library copies every host array it is
 * given; the caller keeps ownership.
 */
#ifndef MHD_GPU_H
#define MHD_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------ */
#define MHD_OK 0
#define MHD_ERR_ARG (-1)      /* bad argument, shape or unsupported option */
#define MHD_ERR_CUDA (-2)     /* CUDA runtime error */
#define MHD_ERR_DT (-3)       /* dt = inf or dt < dtmin (main.c:331) */
#define MHD_ERR_NOMEM (-4)    /* host or device allocation failed */
#define MHD_ERR_STATE (-5)    /* call out of order (e.g. step before upload) */
#define MHD_ERR_TIMEOUT (-6)  /* a bounded device-side wait gave up */
#define MHD_ERR_NODEV (-7)    /* no CUDA device */
#define MHD_ERR_IO (-8)       /* file read/write failed (host I/O helpers) */

/* ---- scheme choices ---------------------------------------------------- */
#define MHD_LIMITER_MINMOD 0  /* MinmodLimiterX/Y/Z (limiterx.h:32, limitery.h:33, limiterz.h:30) */
#define MHD_LIMITER_MC 1      /* MCLimiterX/Y/Z (limiterx.h:335, limitery.h:197, limiterz.h:294) */
#define MHD_LIMITER_VANLEER 2 /* VanLeerLimiterX/Y/Z (limiterx.h:266, limitery.h:129, limiterz.h:232) */
#define MHD_LIMITER_SUPERBEE 3 /* SuperbeeLimiterX/Y/Z (limiterx.h:394, limitery.h:256, limiterz.h:367) */
#define MHD_SOLVER_HLLD 0     /* HLLDX/Y/Z (hlldx.h:28, hlldy.h:30, hlldz.h:28) */
#define MHD_SOLVER_HLL 1      /* HLLX/Y/Z (hllx.h:29, hlly.h:29, hllz.h:26) */
#define MHD_SCHEME_RK2 2      /* live TVDRK: Halfstep + Fullstep (tvdrungekutta.h:31-41) */
#define MHD_SCHEME_RK3 3      /* FirstStep/SecondStep/ThirdStep (tvdrungekutta.h:56-83) */
#define MHD_SOURCE_SPIRAL 0   /* SpiralGravityCooling (source.h:26), the reference's choice */
#define MHD_SOURCE_AXI 1      /* AxiGravityCooling / AxiGravity (source.h:143,207): cooling flag picks */
#define MHD_SOURCE_UNIFORMGZ 2 /* UniformGz (source.h:269): g_z = -1, no geometric terms */
#define MHD_SOURCE_NONE 3     /* NoSource (source.h:308): the geometric terms only */
#define MHD_PREC_FP64 0       /* plain FP64: bit-identical to the reference C */
#define MHD_PREC_FP32 1       /* FP32 state and fluxes, FP64 repair of the fragile steps */
#define MHD_PREC_FP32X2 2     /* MHD_PREC_FP32's FP32 fluxes and primitives, with the conserved state
                                 held as FP32 pairs (hi + lo, about 48 bits): the state no longer rounds
                                 to FP32 every stage.  Split stage shape and thread-load update only
                                 (mhd_set_stage_shape / mhd_set_update_path refuse the others); not in
                                 the batched form. */

/* Physics and scheme knobs.  Reference: input.h:58-96 (#defines and globals),
 * constant.h:62-79.  gamma=5/3 and cr=0.18 are fixed as in constant.h. */
typedef struct {
    double cfl, dtmin, rhocr, prcr, betacr;
    double epssp0, tausp, scalez, scaler, scalephase;
    int armnum;
    double omegasp, omegapattern, pitch;
    int limiter;    /* MHD_LIMITER_* */
    int solver;     /* MHD_SOLVER_* */
    int scheme;     /* MHD_SCHEME_* */
    int cooling;    /* 0 off, 1 Cooling() of cooling.h:22 */
    int gravity;    /* 0 off, 1 Gr*axi + SpiralGravity() each step */
    int precision;  /* MHD_PREC_* */
    int source;     /* MHD_SOURCE_*: the source function the stages call */
} mhd_params;

/* Grid construction parameters (input.h:45-76). */
typedef struct {
    int ix, jy, kz;                   /* interior cells in r, phi, z (jy even) */
    double x0, dx0, lx;               /* first interior r centre, r spacing, stretch start */
    double y0, ly;                    /* first interior phi centre, phi extent */
    double z0, dz0, lz;               /* first interior z centre, z spacing, stretch start */
    double stretchratio, dxmax, dzmax;
    double rin;                       /* central absorbing radius */
} mhd_gridspec;

/* The reference's grid globals (commongrid.h:42-62, commontemp.h:320-322,
 * commonfield.h:130-132), by host pointer in the reference's own layout.
 * ixmax = ix+2 etc.; face-shaped arrays are [ixmax-1][jymax-1][kzmax-1]. */
typedef struct {
    int ix, jy, kz, irin;
    int compact;        /* 0: the reference's 3D layouts below; 1: the j-independent
                           tables g1..g6, minlength, Gr*axi given once per (i,k):
                           g* as [ixmax-1][kzmax-1], the others as [ixmax][kzmax] */
    double dx0, rin;
    const double *x, *xm, *dx, *dxm, *oneox, *oneodx;   /* [ixmax] */
    const double *y;                                     /* [jymax] */
    double dy, oneody;
    const double *z, *zm, *dz, *dzm, *oneodz;           /* [kzmax] */
    const double *g1, *g2, *g3, *g4, *g5, *g6;          /* face-shaped, j-independent */
    const double *minlength;                             /* [ixmax][jymax][kzmax], j-independent */
    double minminlength;
    const double *x_absorb_factor;                       /* [11] */
    const double *z_absorb_factor;                       /* [11] */
    const double *c_absorb_factor;                       /* [irin+1][kzmax] */
    const double *Grxaxi, *Gryaxi, *Grzaxi;              /* [ixmax][jymax][kzmax], j-independent,
                                                            or NULL for zero */
} mhd_grid;

/* Totals over the interior cells, each weighted by the cell volume
 * 0.5*(xm[i]^2-xm[i-1]^2)*dy*dzm[k-1] (cylindricalgrid.h:114), summed in FP64:
 * mass = sum rho dV, angmom = sum (r rho v_phi) dV, energy = sum E dV,
 * psi = sum |psi| dV; maxdivb = max |div B| with central differences
 * (1/r) d(r B_r)/dr + (1/r) dB_phi/dphi + dB_z/dz at interior cells. */
typedef struct {
    double mass, angmom, energy, psi, maxdivb;
} mhd_diag;

typedef struct mhd_ctx mhd_ctx;

/* ---- host helpers (no GPU) ---------------------------------------------- */
const char *mhd_errstr(int code);
void mhd_params_default(mhd_params *p);       /* reference values (input.h, constant.h) */
int mhd_gridspec_disc(int nr, int nphi, int nz, mhd_gridspec *out); /* r in [0.1,1.5], z in [-0.5,0.5] */
int mhd_gridspec_shipped(mhd_gridspec *out);  /* input.h:45-76: 240x64x200 stretched */
/* Doubles of storage mhd_grid_build() needs for the tables. */
size_t mhd_grid_storage(const mhd_gridspec *gs);
/* CylindricalGrid() (cylindricalgrid.h:25-227): fills caller storage and
 * points g's members into it, with compact=1 tables.  Gr*axi are set to NULL. */
int mhd_grid_build(const mhd_gridspec *gs, double *storage, mhd_grid *g);
/* InitialGravity() (initialgravity.h:22-79) into three arrays shaped like
 * g's minlength ([ixmax][kzmax] when compact, else cell-shaped). */
int mhd_initial_gravity(const mhd_grid *g, double *grxaxi, double *gryaxi, double *grzaxi);
/* Project initial condition (no counterpart in the reference): isothermal
 * rotating disc rho = exp(-z^2/(2*0.1^2)) + 1e-3, p = 0.01 rho, v_phi = 1,
 * B_phi = sqrt(2p/beta), with a seeded uniform perturbation of amplitude amp
 * (rho *= 1+amp*u, v += amp*u, u in [-1,1) from splitmix64(seed)).  Writes V,
 * U (VtoU, vtou.h:20-62), Uinit=U, Vinit=V, rhofloor=rhocr*rho
 * (SaveInitial, saveinitial.h:18-50).  Any output pointer may be NULL. */
int mhd_ic_disc(const mhd_grid *g, double beta, double amp, unsigned long long seed,
                double rhocr, double *U, double *V, double *Uinit, double *Vinit,
                double *rhofloor);
/* GalacticDisc3() (model.h:149-327), the reference's shipped initial model:
 * exponential isothermal gas disc + hydrostatic halo in the fixed potential
 * of mhd_initial_gravity(), rotating in the omegasp frame, toroidal field;
 * VtoU, the z=0 symmetry fills of U, SaveInitial.  Pair it with
 * mhd_gridspec_shipped() and mhd_initial_gravity() (the potential it assumes).
 * Uinit, Vinit, rhofloor may be NULL. */
int mhd_ic_galactic_disc3(const mhd_grid *g, const mhd_params *p, double *U, double *V, double *Uinit,
                          double *Vinit, double *rhofloor);
/* VtoU() (vtou.h:20-62) on caller arrays. */
int mhd_vtou(const mhd_grid *g, const double *V, double *U);

/* ---- checkpoint files and restart (host, no GPU) ------------------------ */
/* BinaryOutput() (output.h:1202-1414): directory <root>/<nout> holding
 * GridTime.dat (text "%d\t%d\t%d\t%.3e" of ixmax, jymax, kzmax, t), the cell
 * centres r, phi, z and V as raw FP64 files rho vr vphi vz br bphi bz pr psi,
 * each [ixmax][jymax][kzmax] with ghosts.  root "." is the reference's own
 * location.  The _arrays form takes the dimensions and the centre arrays. */
int mhd_binary_output(const char *root, int nout, double t, const mhd_grid *g, const double *V);
int mhd_binary_output_arrays(const char *root, int nout, double t, int ix, int jy, int kz, const double *x,
                             const double *y, const double *z, const double *V);
/* The file part of RestartRead() (restartread.h:9-121): V from <root>/<num>. */
int mhd_restart_read(const char *root, int num, int ix, int jy, int kz, double *V);
/* Check() (check.h:23-188) on caller arrays, every cell: density, pressure
 * and plasma-beta floors; counters (may be NULL) = cells caught by each. */
int mhd_check(const mhd_grid *g, const mhd_params *p, double *U, double *V, const double *rhofloor,
              int counters[3]);
/* SaveInitial() (saveinitial.h:18-50): Uinit=U, Vinit=V, rhofloor=rhocr*rho. */
int mhd_save_initial(const mhd_grid *g, double rhocr, const double *U, const double *V, double *Uinit,
                     double *Vinit, double *rhofloor);
/* The restart branch of main.c:244-270: RestartRead(0) (VtoU + Check with
 * zero floors), SaveInitial(), RestartRead(nout); t = nout*tint and
 * tout = (nout+1)*tint.  Gravity tables are the caller's (InitialGravity). */
int mhd_restart(const char *root, int nout, double tint, const mhd_grid *g, const mhd_params *p, double *U,
                double *V, double *Uinit, double *Vinit, double *rhofloor, double *t, double *tout);

/* Text outputs for plotting, the reference's formats, written under root:
 * GNUOutputCylinder (output.h:25-150): 1d-r-<nout>.dat (j=1, k=1),
 * 1d-phi-<nout>.dat and 1d-z-<nout>.dat at the radial index 160 the
 * reference fixes (MHD_ERR_ARG when ix < 159); columns coordinate, rho, v_r,
 * v_phi, v_z, B_r, B_phi, B_z, E (= U[7]), p.  GDLOutputCylinder
 * (output.h:280-390): r.dat, phi.dat, z.dat, the k=1 slices
 * 2d-{density,pressure,benergy}-rphi-<nout>.dat and 2d-density-rz-<nout>.dat. */
int mhd_gnu_output_cylinder(const char *root, int nout, int nstep, double t, const mhd_grid *g, const double *U,
                            const double *V);
int mhd_gdl_output_cylinder(const char *root, int nout, const mhd_grid *g, const double *V);

/* ---- device context: the step ------------------------------------------- */
/* A context binds the calling thread's current CUDA device at mhd_create().
 * mhd_use_device() makes device `ordinal` (0-based among the visible devices)
 * current for the calling thread -- one process per GPU calls it with its
 * local rank before its first mhd_create(); MHD_ERR_ARG for an ordinal
 * outside [0, device count), MHD_ERR_NODEV without a CUDA device.
 * mhd_current_device() returns the calling thread's current ordinal. */
int mhd_use_device(int ordinal);
int mhd_current_device(int *ordinal);
int mhd_create(const mhd_grid *g, const mhd_params *p, mhd_ctx **out);
void mhd_destroy(mhd_ctx *ctx);
/* State upload, host layout [9][ixmax][jymax][kzmax] FP64 (commonfield.h:114,
 * commontemp.h:305-308).  Uinit/Vinit/rhofloor feed the absorbing layers, the
 * MC z boundary and the density floor; NULL means "same as U", "same as V"
 * and rhocr*U[0] (SaveInitial, saveinitial.h:34-40) respectively. */
int mhd_upload(mhd_ctx *ctx, const double *U, const double *V, const double *Uinit,
               const double *Vinit, const double *rhofloor);
int mhd_download(mhd_ctx *ctx, double *U, double *V);
/* Setdt (setdt.h:24-94): dt = cfl/max, ch = minminlength*max; ijk = the
 * first cell (in i,j,k order) attaining the max, as the serial reference. */
int mhd_setdt(mhd_ctx *ctx, double *dt, double *ch, int ijk[3]);
/* SpiralGravity (spiralgravity.h:20-124) at time t: takes effect for the
 * following mhd_tvdrk(). */
int mhd_spiral_gravity(mhd_ctx *ctx, double t);
/* TVDRK (tvdrungekutta.h:16-78) with the given dt and ch; counters = the
 * density, pressure and beta floor counts of the last stage's Check
 * (check.h:180-183). */
int mhd_tvdrk(mhd_ctx *ctx, double dt, double ch, int counters[3]);
/* One pass of main.c:319-351: Setdt, dt guard, SpiralGravity (if gravity),
 * TVDRK, t += dt.  Returns MHD_ERR_DT (state untouched) where the reference
 * exits. */
int mhd_step(mhd_ctx *ctx, double *t, double *dt, double *ch, int counters[3]);
/* nsteps of mhd_step with no host round trip: dt, ch and the psi factor stay
 * on the device and the whole step is one CUDA graph launch.  Only for
 * MHD_PREC_FP32 (the plain form computes exp() on the host for bitwise
 * parity).  *t advances by the sum of the dt's. */
int mhd_run(mhd_ctx *ctx, int nsteps, double *t);
int mhd_diagnostics(mhd_ctx *ctx, mhd_diag *d);
/* The CUDA stream the context launches on (as a cudaStream_t). */
void *mhd_stream(mhd_ctx *ctx);
/* Upload only the evolving state U, V (same layout as mhd_upload); the
 * initial arrays and floors from the last mhd_upload stay.  V = NULL: the
 * primitives are formed on the device as UtoV(U) (utov.h:24-68) at every cell,
 * which halves the bytes a host that keeps only the conserved state moves
 * (with mhd_download(ctx, U, NULL) on the way back).  Where Check's floors
 * fired in the step that produced U, UtoV(U) differs from the V that step
 * stored by rounding, so the plain form is then no longer bit-identical to a
 * reference run that kept V. */
int mhd_upload_state(mhd_ctx *ctx, const double *U, const double *V);

/* Asynchronous BinaryOutput of the context's current V: the state is copied
 * (as FP64) to a device snapshot on the context's stream, then to pinned host
 * memory on a second stream, and a host thread writes <root>/<nout> once the
 * copy lands -- the caller keeps stepping meanwhile.  One checkpoint is in
 * flight at a time: begin waits for the previous one.  wait returns the
 * writer's status (MHD_ERR_IO on a failed write).  Device and pinned memory
 * for the snapshot (9 FP64 arrays each) are taken on the first call. */
int mhd_checkpoint_begin(mhd_ctx *ctx, const char *root, int nout, double t);
int mhd_checkpoint_wait(mhd_ctx *ctx);

/* ---- instrumentation ------------------------------------------------------ */
/* Per-kernel timing with CUDA events recorded around every launch on the
 * context's stream (off by default; enabling resets the totals).  Kinds:
 * 0 flux r, 1 flux phi, 2 flux z, 3 update, 4 ghost fill, 5 CFL reduction,
 * 6 arm-phase table, 7 state conversion, 8 fused stage (fluxes + update),
 * 9 z fluxes + update. */
#define MHD_PROF_NKIND 10
int mhd_prof_enable(mhd_ctx *ctx, int on);
int mhd_prof_read(mhd_ctx *ctx, double ms[MHD_PROF_NKIND], long long launches[MHD_PROF_NKIND]);
/* How a stage runs.  fused = 0: three flux kernels write F, G, H to device
 * memory and an update kernel reads them; fused = 2: the r and phi flux
 * kernels, then one kernel forms the z fluxes in registers and updates the
 * cells; fused = 1: one kernel forms all fluxes on chip and updates the cells
 * (tile 32 k-cells x tj j-cells, tj = 7, marching over runs of seg cells in
 * r); fused = 3: the kernels of fused = 0 pipelined over seg slabs of i
 * planes (1..64; tj ignored), the update of each slab on a second,
 * higher-priority stream beside the fluxes of the next slabs.  All give the
 * same bits in the plain form. */
int mhd_set_stage_shape(mhd_ctx *ctx, int fused, int tj, int seg);
/* How the split stage's update reads its inputs (precision form): tma = 0
 * (the default) loads them thread by thread; tma = 1 stages each tile of 128
 * cells in shared memory with tensor copies, where the layout allows it
 * (cells per variable a multiple of 4).  MHD_ERR_ARG for tma = 1 where it is
 * not available (plain form, other layouts); tma = 2 (precision form) keeps
 * the thread loads and has each block prefetch the streamed inputs of the
 * block one wave of resident blocks ahead into L2.  With tma = 1, a tile
 * whose copies do not land within a bounded wait makes the step return
 * MHD_ERR_TIMEOUT.  That
 * give-up path waits a second bounded time for the copies still in flight;
 * should that wait also run out, the block exits with bulk copies possibly
 * still writing its shared memory, which is unsafe -- the option stays off
 * by default, and no test drives either wait to its limit. */
int mhd_set_update_path(mhd_ctx *ctx, int tma);
/* Precision diagnostic of the plain form: with on = 1 the arithmetic stays
 * FP64 but every stage stores U and V rounded to FP32, as a form with FP32
 * state must -- a run of it (from an FP32-rounded start) measures the error
 * that FP32 storage alone causes, the floor of MHD_PREC_FP32's error against
 * the plain form.  MHD_ERR_ARG on a precision-form context. */
int mhd_set_state_rounding(mhd_ctx *ctx, int on);
/* The split stage's update path set by mhd_set_update_path (0, 1 or 2). */
int mhd_update_path(const mhd_ctx *ctx);
/* Kernels this context has launched since creation. */
long long mhd_launch_count(const mhd_ctx *ctx);
/* Stream timer: start synchronises the stream and records an event; stop
 * records a second event, waits for it and returns the elapsed device time. */
int mhd_timer_start(mhd_ctx *ctx);
int mhd_timer_stop(mhd_ctx *ctx, double *ms);
/* Page-lock (on=1) or release (on=0) a caller's host buffer so the
 * context's copies from/to it run asynchronously at full link speed. */
int mhd_pin(void *ptr, size_t bytes, int on);

/* ---- per-kernel probes (parity tests) ------------------------------------ */
/* Reconstructed face states of one direction (dir 0 r, 1 phi, 2 z) with the
 * given dt, in the reference's face layout [9][ixmax-1][jymax-1][kzmax-1];
 * entries the step never reads are left zero. */
int mhd_dbg_limiter(mhd_ctx *ctx, int dir, double dt, double *Vl, double *Vr);
/* Riemann flux + GLM flux of one direction (F, G or H) in the face layout. */
int mhd_dbg_flux(mhd_ctx *ctx, int dir, double dt, double ch, double *F);
/* SpiralGravityCooling source S (source.h:26-134), cell layout [9][...]. */
int mhd_dbg_source(mhd_ctx *ctx, double *S);
/* Grx, Gry, Grz of the last mhd_spiral_gravity(), cell layout [3][...]. */
int mhd_dbg_gravity(mhd_ctx *ctx, double *gr);

/* ---- batched form: many independent discs ------------------------------- */
typedef struct mhd_batch mhd_batch;
/* One precision (MHD_PREC_FP64 or MHD_PREC_FP32; MHD_PREC_FP32X2 is refused
 * with MHD_ERR_ARG) and one RK scheme for all n discs. */
int mhd_batch_create(int n, const mhd_grid *grids, const mhd_params *params, mhd_batch **out);
void mhd_batch_destroy(mhd_batch *b);
int mhd_batch_upload(mhd_batch *b, int disc, const double *U, const double *V,
                     const double *Uinit, const double *Vinit, const double *rhofloor);
int mhd_batch_download(mhd_batch *b, int disc, double *U, double *V);
/* nsteps steps of every disc, each with its own dt; t[n] advance in place;
 * status[n] = 0 or MHD_ERR_DT for a disc whose dt guard fired (that disc then
 * stops advancing).  The whole step is one CUDA graph launch.  Precision form:
 * by default one persistent launch per RK stage over a work queue of all
 * discs (r, phi and z flux items and update items per slab of r planes,
 * ghost items; an update slab waits, bounded, for the flux items of its slab
 * and the one below); mhd_batch_tune() may pick the phased or disc-graph
 * mode instead.  Plain form: the discs' mhd_step() one after another. */
int mhd_batch_step(mhd_batch *b, int nsteps, double *t, int *status);
/* Times candidate configurations on the current state and keeps the fastest;
 * the state is restored afterwards.  Candidates: the persistent per-stage
 * launch with each of 8 configurations (mode 0: slab depth 8, 16 or 32 r
 * planes, queue lag 1 or 2 slabs, register cap 102 or 128 per thread), the
 * phased form -- one launch per stage phase over all discs (mode 1) -- and
 * the disc graph -- every disc's own single-disc step, the discs dealt to 2,
 * 4, 8 or 16 parallel stream branches of one graph (mode 2).
 * best[5] = {slab planes, queue lag, registers per thread, threads, 0} for
 * mode 0; {1, 1, 128, 128, 1} for mode 1; {branches, 0, 0, 0, 2} for mode 2. */
int mhd_batch_tune(mhd_batch *b, int *best);
/* Pick the precision form's batch mode directly: 0 persistent with
 * configuration arg (0..7, the tuner's order), 1 phased, 2 disc graph on arg
 * branches (1..64). */
int mhd_batch_set_mode(mhd_batch *b, int mode, int arg);
/* Test hook for the persistent mode's bounded waits (an update item waits,
 * with an iteration limit, for its slab's flux items): with disc >= 0 the
 * flux count that disc's first slab waits for is set one above what the
 * stage produces and the limit
 * to spin_limit, so the next step's wait runs out -- no fault, no hang -- and
 * mhd_batch_step returns MHD_ERR_TIMEOUT (the state of that step is then
 * undefined: upload again).  disc = -1 restores normal operation.  Selects
 * the persistent mode. */
int mhd_batch_debug_stall(mhd_batch *b, int disc, int spin_limit);

/* ---- allocation-free CFL reduction -------------------------------------- */
/* No counterpart in the reference.  For callers that may not call cudaMalloc
 * when they need a step size (a host that hands out device memory from its own
 * pool and forbids allocation afterwards, a real-time loop): the same CFL
 * reduction as mhd_setdt(), with its scratch in a fixed device array of
 * MHD_NOALLOC_MAX_BLOCKS partials (about 128 KB, held by every GPU that loads
 * the library until exit) instead of a context buffer; it allocates nothing.
 * Inputs are device pointers: V [9][ix+2][jy+2][kz+2] FP64 and minlength
 * [ix+2][kz+2]; dt, ch, ijk are host outputs as for mhd_setdt().  Grids whose
 * CFL range (ix-10)*jy*kz exceeds MHD_NOALLOC_MAX_BLOCKS*256*64 cells
 * (134,217,728) are rejected with MHD_ERR_ARG before any launch.  The first
 * call on a device looks up the array's device address and caches it for the
 * process; with CUDA's default lazy module loading that first call may also
 * be what loads this code onto the device and maps the array, so make it at
 * start-up, before the no-allocation window opens and before any stream
 * capture.  The cached address does not survive a device reset
 * (cudaDeviceReset or a torn-down primary context): calling again after one
 * is not supported.  Calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller. */
#define MHD_NOALLOC_MAX_BLOCKS 8192
int mhd_setdt_noalloc(const double *V, const double *minlength, int ix, int jy, int kz, double cfl,
                      double minminlength, int cooling, void *stream, double *dt, double *ch, int ijk[3]);

#ifdef __cplusplus
}
#endif
#endif
