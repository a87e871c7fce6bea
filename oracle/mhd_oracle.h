/*
 * mhd_oracle.h -- CPU restatement of the reference's cylindrical GLM-MHD
 * TVD Runge-Kutta step (test infrastructure: the ORACLE, never the product).
 *
 * Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
 * legs may load this library, and only as the checker or the CPU baseline.
 *
 * It restates, with run-time grid sizes, every function on the reference's
 * step path with the reference's loop order and expression order, so that a
 * run reproduces the reference C bit for bit (pinned in this repository's CPU
 * tests against the reference compiled in place, and against committed golden
 * vectors made from it).  Each function cites the reference file:line it
 * follows.  Arrays use the reference's layout [m][i][j][k] (k fastest); face
 * arrays use the cell-array shape here (ixmax x jymax x kzmax) instead of the
 * reference's (ixmax-1) x (jymax-1) x (kzmax-1).
 */
#ifndef MHD_ORACLE_H
#define MHD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Grid description (reference input.h:45-76 and cylindricalgrid.h:36-102). */
typedef struct {
    int nr, nphi, nz;          /* ix, jy, kz: interior cells */
    double x0, dx0, lx;        /* first interior r centre, r spacing, stretch start */
    double y0, ly;             /* first interior phi centre, phi extent */
    double z0, dz0, lz;        /* first interior z centre, z spacing, stretch start */
    double stretchratio, dxmax, dzmax;
    double rin;                /* central absorbing radius */
} orc_gridspec;

/* Physics and scheme knobs (reference input.h:58-96, constant.h:62-79). */
typedef struct {
    double cfl, dtmin, rhocr, prcr, betacr;
    double epssp0, tausp, scalez, scaler, scalephase, armnum;
    double omegasp, omegapattern, pitch;
    int limiter;   /* 0 minmod (limiterx.h:32), 1 MC (limiterx.h:335), 2 van Leer (:266), 3 superbee (:394) */
    int solver;    /* 0 HLLD (hlldx.h:28), 1 HLL (hllx.h:29) */
    int scheme;    /* 2 live RK2 (halfstep/fullstep), 3 RK3 (first/second/thirdstep) */
    int cooling;   /* 0 off, 1 cooling.h:22 */
    int gravity;   /* 0 off, 1 axisymmetric + spiral (initialgravity.h, spiralgravity.h) */
    int source;    /* 0 SpiralGravityCooling, 1 AxiGravity(Cooling), 2 UniformGz, 3 NoSource (source.h) */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_gridspec *gs, const orc_params *p);
void orc_destroy(orc_ctx *o);
void orc_dims(const orc_ctx *o, int *out7);   /* ix jy kz ixmax jymax kzmax irin */
void orc_set_threads(int n);

/* grid tables (each of length ixmax / jymax / kzmax; scalars: dy, oneody,
 * minminlength, oneominminlength) */
void orc_get_grid1d(const orc_ctx *o, double *x, double *xm, double *dx, double *dxm,
                    double *oneox, double *oneoxm, double *oneodx, double *y, double *z,
                    double *zm, double *dz, double *dzm, double *oneodz, double *scalars);
/* g1..g6 in the reference face layout [6][ixmax-1][jymax-1][kzmax-1], minlength
 * [ixmax][jymax][kzmax], absorbing factors x[11], z[11], c[irin+1][kzmax], krin */
void orc_get_metric(const orc_ctx *o, double *g, double *minlen, double *xabs,
                    double *zabs, double *cabs, int *krin);

void orc_initial_gravity(orc_ctx *o);                 /* initialgravity.h:22 */
void orc_set_gravity_axi(orc_ctx *o, const double *axi); /* [3][cells] */
void orc_get_gravity(const orc_ctx *o, double *axi, double *gr);

void orc_load(orc_ctx *o, const double *U, const double *V, const double *Uinit,
              const double *Vinit, const double *rhofloor);
void orc_store(const orc_ctx *o, double *U, double *V, double *U1);
/* the benchmark's seeded disc (V, U, Uinit, Vinit, rhofloor) set in place */
void orc_ic_disc(orc_ctx *o, double beta, double amp, unsigned long long seed);

void orc_setdt(orc_ctx *o, double *dt, double *ch, int *ijk);   /* setdt.h:24 */
void orc_spiral_gravity(orc_ctx *o, double t);                 /* spiralgravity.h:20 */
/* one step of main.c:319-351; returns 1 when the dt guard of main.c:331 fires */
int orc_step(orc_ctx *o, double *t, double *dt, double *ch, int *counters);

/* per-kernel probes (face outputs in the reference face layout) */
void orc_set_dtch(orc_ctx *o, double dt, double ch, double psicoef);
void orc_limiter(orc_ctx *o, int dir, double *Vl, double *Vr);
void orc_flux(orc_ctx *o, int dir, double *F);
void orc_source(orc_ctx *o, double *S);
void orc_utov_check(orc_ctx *o, double *U, double *V, int *counters);
int orc_cooling(double rho, double pr);

#ifdef __cplusplus
}
#endif
#endif
