/*
 * mhd_host.c -- host-side helpers of libmhdgpu.so: reference defaults, grid
 * construction, axisymmetric gravity and the project initial condition.
 *
 * These run once at set-up on the CPU, exactly where the reference runs them
 * (CylindricalGrid() and GalacticDisc3()/InitialGravity() before the step
 * loop, main.c:232,277,299).  They use the host C library's math so the
 * tables the kernels read are the values the reference computes.  Compiled
 * with -ffp-contract=off: no multiply-add contraction, on x86 or Arm.
 */
#include "mhd_gpu.h"
#include "mhd_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

const char *mhd_errstr(int code)
{
    switch (code) {
    case MHD_OK: return "ok";
    case MHD_ERR_ARG: return "bad argument or shape";
    case MHD_ERR_CUDA: return "CUDA runtime error";
    case MHD_ERR_DT: return "stop due to small dt or inf (dt guard)";
    case MHD_ERR_NOMEM: return "out of memory";
    case MHD_ERR_STATE: return "call out of order";
    case MHD_ERR_TIMEOUT: return "bounded device wait expired";
    case MHD_ERR_NODEV: return "no CUDA device";
    case MHD_ERR_IO: return "file I/O failed";
    default: return "unknown error";
    }
}

/* input.h:58-96 and constant.h:47-89 */
void mhd_params_default(mhd_params *p)
{
    const double year = 3.1536e+7, t0 = 4.7058e+15, kpc = 3.08568e+21;
    const double omega0 = (1.0 / t0), oneokpc = (1.0 / kpc);
    memset(p, 0, sizeof *p);
    p->cfl = 0.4;
    p->dtmin = 1.0e-9;
    p->rhocr = 1.0e-4;
    p->prcr = 0.015;
    p->betacr = 0.1;
    p->epssp0 = 0.05;
    p->tausp = 200.0 * 1.0e+6 * year / t0;
    p->scalez = 0.03;
    p->scaler = 0.7;
    p->scalephase = 0.1;
    p->armnum = 2;
    p->omegasp = 10.0e+5 / omega0 * oneokpc;
    p->omegapattern = 10.0e+5 / omega0 * oneokpc;
    p->pitch = 15.0 * M_PI / 180.0;
    p->limiter = MHD_LIMITER_MINMOD;
    p->solver = MHD_SOLVER_HLLD;
    p->scheme = MHD_SCHEME_RK2;
    p->cooling = 1;
    p->gravity = 1;
    p->precision = MHD_PREC_FP64;
}

int mhd_gridspec_disc(int nr, int nphi, int nz, mhd_gridspec *s)
{
    if (!s || nr < 12 || nz < 12 || nphi < 4 || (nphi & 1)) return MHD_ERR_ARG;
    memset(s, 0, sizeof *s);
    s->ix = nr; s->jy = nphi; s->kz = nz;
    s->dx0 = 1.4 / (double)nr;
    s->x0 = (0.1 + 0.5 * s->dx0);
    s->lx = 1.0e30;
    s->y0 = 0.0;
    s->ly = 2.0 * M_PI;
    s->dz0 = 1.0 / (double)nz;
    s->z0 = (-0.5 + 0.5 * s->dz0);
    s->lz = 1.0e30;
    s->stretchratio = 1.05;
    s->dxmax = 50.0 * s->dx0;
    s->dzmax = 50.0 * s->dz0;
    s->rin = 0.1;
    return MHD_OK;
}

/* input.h:45-76 as shipped */
int mhd_gridspec_shipped(mhd_gridspec *s)
{
    if (!s) return MHD_ERR_ARG;
    memset(s, 0, sizeof *s);
    s->ix = 240; s->jy = 64; s->kz = 200;
    s->lx = 2.0; s->ly = 2.0 * M_PI; s->lz = 0.03;
    s->x0 = 0.04; s->y0 = 0.0; s->z0 = 0.0;
    s->stretchratio = 1.05;
    s->rin = 0.1;
    s->dx0 = 0.01; s->dz0 = 0.0003;
    s->dxmax = 50.0 * s->dx0;
    s->dzmax = 50.0 * s->dz0;
    return MHD_OK;
}

static int irin_of(const mhd_gridspec *s) { return (int)(s->rin / s->dx0); }

size_t mhd_grid_storage(const mhd_gridspec *s)
{
    size_t ixm = (size_t)s->ix + 2, jym = (size_t)s->jy + 2, kzm = (size_t)s->kz + 2;
    return 6 * ixm + jym + 5 * kzm + 6 * (ixm - 1) * (kzm - 1) + ixm * kzm + 22
           + ((size_t)irin_of(s) + 1) * kzm;
}

static double dmin(double a, double b) { return a > b ? b : a; }   /* maxmin.h:22 */

/* cylindricalgrid.h:25-227 */
int mhd_grid_build(const mhd_gridspec *s, double *st, mhd_grid *g)
{
    if (!s || !st || !g || s->ix < 12 || s->kz < 12 || s->jy < 4 || (s->jy & 1) || s->dx0 <= 0.0)
        return MHD_ERR_ARG;
    int ixmax = s->ix + 2, jymax = s->jy + 2, kzmax = s->kz + 2;
    int ixmax1 = ixmax - 1, jymax1 = jymax - 1, kzmax1 = kzmax - 1;
    int irin = irin_of(s);
    if (irin < 0 || irin + 1 > ixmax) return MHD_ERR_ARG;
    memset(g, 0, sizeof *g);
    g->ix = s->ix; g->jy = s->jy; g->kz = s->kz; g->irin = irin; g->compact = 1;
    g->dx0 = s->dx0; g->rin = s->rin;

    double *x = st; st += ixmax;
    double *xm = st; st += ixmax;
    double *dx = st; st += ixmax;
    double *dxm = st; st += ixmax;
    double *oneox = st; st += ixmax;
    double *oneodx = st; st += ixmax;
    double *y = st; st += jymax;
    double *z = st; st += kzmax;
    double *zm = st; st += kzmax;
    double *dz = st; st += kzmax;
    double *dzm = st; st += kzmax;
    double *oneodz = st; st += kzmax;
    size_t gsz = (size_t)ixmax1 * kzmax1;
    double *gt[6];
    for (int n = 0; n < 6; n++) { gt[n] = st; st += gsz; }
    double *minlength = st; st += (size_t)ixmax * kzmax;
    double *xabs = st; st += 11;
    double *zabs = st; st += 11;
    double *cabs = st; st += (size_t)(irin + 1) * kzmax;

    /* r (cylindricalgrid.h:36-65) */
    dx[0] = s->dx0;
    x[0] = s->x0 - s->dx0;
    for (int i = 0; i < ixmax1; i++) {
        x[i + 1] = x[i] + dx[i];
        dx[i + 1] = (x[i] > s->lx) ? dmin(s->stretchratio * dx[i], s->dxmax) : dx[i];
        xm[i] = (x[i] + x[i + 1]) * 0.5;
        dxm[i] = (dx[i] + dx[i + 1]) * 0.5;
        oneox[i] = 1.0 / x[i];
        oneodx[i] = 1.0 / dx[i];
    }
    xm[ixmax1] = x[ixmax1] + 0.5 * dx[ixmax1];
    dxm[ixmax1] = dx[ixmax1];
    oneox[ixmax1] = 1.0 / x[ixmax1];
    oneodx[ixmax1] = 1.0 / dx[ixmax1];

    /* phi (cylindricalgrid.h:70-74) */
    double dy = s->ly / (double)s->jy;
    y[0] = s->y0 - dy;
    for (int j = 0; j < jymax1; j++) y[j + 1] = y[j] + dy;

    /* z (cylindricalgrid.h:79-102) */
    dz[0] = s->dz0;
    z[0] = s->z0 - s->dz0;
    for (int k = 0; k < kzmax1; k++) {
        z[k + 1] = z[k] + dz[k];
        dz[k + 1] = (z[k] > s->lz) ? dmin(s->stretchratio * dz[k], s->dzmax) : dz[k];
        zm[k] = (z[k] + z[k + 1]) * 0.5;
        dzm[k] = (dz[k] + dz[k + 1]) * 0.5;
        oneodz[k] = 1.0 / dz[k];
    }
    zm[kzmax1] = z[kzmax1] + 0.5 * dz[kzmax1];
    oneodz[kzmax1] = 1.0 / dz[kzmax1];

    /* geometric factors (cylindricalgrid.h:108-130), identical for every j */
    for (size_t q = 0; q < 6 * gsz; q++) gt[0][q] = 0.0;
    for (int i = 1; i < ixmax1; i++)
        for (int k = 1; k < kzmax1; k++) {
            double dvolume = 0.5 * (xm[i] * xm[i] - xm[i - 1] * xm[i - 1]) * dy * dzm[k - 1];
            double oneodvol = 1.0 / dvolume;
            size_t q = (size_t)i * kzmax1 + k;
            gt[0][q] = xm[i - 1] * dy * dzm[k - 1] * oneodvol;
            gt[1][q] = xm[i] * dy * dzm[k - 1] * oneodvol;
            gt[2][q] = dxm[i - 1] * dzm[k - 1] * oneodvol;
            gt[3][q] = gt[2][q];
            gt[4][q] = 0.5 * (xm[i] * xm[i] - xm[i - 1] * xm[i - 1]) * dy * oneodvol;
            gt[5][q] = gt[4][q];
        }

    /* minimum cell length (cylindricalgrid.h:136-163) */
    double oneominminlength = 0.0;
    for (int i = 0; i < ixmax; i++)
        for (int k = 0; k < kzmax; k++) {
            double ml = dmin(dx[i], dmin(x[i] * dy, dz[k]));
            minlength[(size_t)i * kzmax + k] = ml;
            double inv = 1.0 / ml;
            if (inv > oneominminlength) oneominminlength = inv;
        }

    /* absorbing factors (cylindricalgrid.h:168-201) */
    for (int i = ixmax1 - 10; i < ixmax; i++)
        xabs[i - (ixmax1 - 10)] = (0.5 * (1.0 - tanh((x[ixmax1] - x[i] - 5.0 * dx[ixmax1]) / (2.0 * dx[ixmax1]))));
    for (int k = kzmax1 - 10; k < kzmax; k++)
        zabs[k - (kzmax1 - 10)] = (0.5 * (1.0 - tanh((z[kzmax1] - z[k] - 5.0 * dz[kzmax1]) / (2.0 * dz[kzmax1]))));
    for (int i = 0; i < irin + 1; i++)
        for (int k = 0; k < kzmax; k++) {
            double r = sqrt(x[i] * x[i] + z[k] * z[k]);
            cabs[(size_t)i * kzmax + k] = (0.5 * (1.0 - tanh((r - s->rin + 5.0 * s->dx0) / (2.0 * s->dx0))));
        }

    g->x = x; g->xm = xm; g->dx = dx; g->dxm = dxm; g->oneox = oneox; g->oneodx = oneodx;
    g->y = y; g->dy = dy; g->oneody = 1.0 / dy;
    g->z = z; g->zm = zm; g->dz = dz; g->dzm = dzm; g->oneodz = oneodz;
    g->g1 = gt[0]; g->g2 = gt[1]; g->g3 = gt[2]; g->g4 = gt[3]; g->g5 = gt[4]; g->g6 = gt[5];
    g->minlength = minlength;
    g->minminlength = 1.0 / oneominminlength;
    g->x_absorb_factor = xabs; g->z_absorb_factor = zabs; g->c_absorb_factor = cabs;
    g->Grxaxi = g->Gryaxi = g->Grzaxi = NULL;
    return MHD_OK;
}

/* The fixed axisymmetric potential's parameters (initialgravity.h:34-36,
 * model.h:162-164): logarithmic dark halo (vhalo0, dh), Miyamoto-Nagai disc
 * (a, b, md), Hernquist bulge (db, mb); v0 = 6.558e+6 (constant.h:84). */
static const double GV_VHALO0 = 131.5e+5 / 6.558e+6, GV_DH = 1.2;
static const double GV_A = 0.65, GV_B = 0.026, GV_MD = 10.0;
static const double GV_DB = 0.07, GV_MB = 3.4;

/* radial and vertical axisymmetric gravity at (x, z): initialgravity.h:52-70,
 * model.h:229-246 (the two spell the same expressions) */
static double axi_grx(double x, double z)
{
    const double vhalo0 = GV_VHALO0, dh = GV_DH, a = GV_A, b = GV_B, md = GV_MD, db = GV_DB, mb = GV_MB;
    double x2 = x * x, z2 = z * z;
    return ((-2.0 * vhalo0 * vhalo0 / (x2 + z2 + dh * dh)
             - md / pow(x2 + (a + sqrt(z2 + b * b)) * (a + sqrt(z2 + b * b)), 1.5)
             - mb / ((sqrt(x2 + z2) + db) * (sqrt(x2 + z2) + db) * sqrt(x2 + z2)))
            * x);
}

static double axi_grz(double x, double z)
{
    const double vhalo0 = GV_VHALO0, dh = GV_DH, a = GV_A, b = GV_B, md = GV_MD, db = GV_DB, mb = GV_MB;
    double x2 = x * x, z2 = z * z;
    return ((-2.0 * vhalo0 * vhalo0 / (x2 + z2 + dh * dh)
             - md / pow(x2 + (a + sqrt(z2 + b * b)) * (a + sqrt(z2 + b * b)), 1.5)
               * (1.0 + a / sqrt(z2 + b * b))
             - mb / ((sqrt(x2 + z2) + db) * (sqrt(x2 + z2) + db) * sqrt(x2 + z2)))
            * z);
}

/* initialgravity.h:22-79 */
int mhd_initial_gravity(const mhd_grid *g, double *grx, double *gry, double *grz)
{
    if (!g || !grx || !gry || !grz) return MHD_ERR_ARG;
    int ixmax = g->ix + 2, jymax = g->jy + 2, kzmax = g->kz + 2;
    int nj = g->compact ? 1 : jymax;
    for (int i = 0; i < ixmax; i++)
        for (int j = 0; j < nj; j++)
            for (int k = 0; k < kzmax; k++) {
                size_t q = ((size_t)i * nj + j) * kzmax + k;
                grx[q] = axi_grx(g->x[i], g->z[k]);
                gry[q] = 0.0;
                grz[q] = axi_grz(g->x[i], g->z[k]);
            }
    return MHD_OK;
}

/* VtoU (vtou.h:27-57) for one cell */
static void cell_vtou(const double *v, size_t nc, size_t q, double xi, double *U)
{
    double v0 = v[q], v1 = v[nc + q], v2v = v[2 * nc + q], v3 = v[3 * nc + q];
    double v4 = v[4 * nc + q], v5 = v[5 * nc + q], v6 = v[6 * nc + q];
    double v2 = v1 * v1 + v2v * v2v + v3 * v3;
    double b2 = v4 * v4 + v5 * v5 + v6 * v6;
    U[q] = v0;
    U[nc + q] = v0 * v1;
    U[2 * nc + q] = xi * v0 * v2v;
    U[3 * nc + q] = v0 * v3;
    U[4 * nc + q] = v4;
    U[5 * nc + q] = v5;
    U[6 * nc + q] = v6;
    U[7 * nc + q] = 0.5 * (v0 * v2 + b2) + 1.5 * v[7 * nc + q];
    U[8 * nc + q] = v[8 * nc + q];
}

int mhd_vtou(const mhd_grid *g, const double *V, double *U)
{
    if (!g || !V || !U) return MHD_ERR_ARG;
    size_t ixmax = (size_t)g->ix + 2, jymax = (size_t)g->jy + 2, kzmax = (size_t)g->kz + 2;
    size_t nc = ixmax * jymax * kzmax;
    for (size_t i = 0; i < ixmax; i++)
        for (size_t q = i * jymax * kzmax; q < (i + 1) * jymax * kzmax; q++)
            cell_vtou(V, nc, q, g->x[i], U);
    return MHD_OK;
}

static unsigned long long splitmix64(unsigned long long *s)
{
    unsigned long long z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* uniform in [-1, 1) */
static double unit_pm(unsigned long long *s)
{
    return 2.0 * ((double)(splitmix64(s) >> 11) * 0x1.0p-53) - 1.0;
}

int mhd_ic_disc(const mhd_grid *g, double beta, double amp, unsigned long long seed,
                double rhocr, double *U, double *V, double *Uinit, double *Vinit, double *rhofloor)
{
    if (!g || beta <= 0.0) return MHD_ERR_ARG;
    size_t ixmax = (size_t)g->ix + 2, jymax = (size_t)g->jy + 2, kzmax = (size_t)g->kz + 2;
    size_t nc = ixmax * jymax * kzmax;
    double *Vw = V ? V : (double *)malloc(9 * nc * sizeof(double));
    if (!Vw) return MHD_ERR_NOMEM;
    unsigned long long st = seed;
    for (size_t i = 0; i < ixmax; i++)
        for (size_t j = 0; j < jymax; j++)
            for (size_t k = 0; k < kzmax; k++) {
                size_t q = (i * jymax + j) * kzmax + k;
                double zk = g->z[k];
                double rho = exp(-zk * zk / (2.0 * 0.1 * 0.1)) + 1.0e-3;
                double ur = unit_pm(&st), uvr = unit_pm(&st), uvp = unit_pm(&st), uvz = unit_pm(&st);
                rho = rho * (1.0 + amp * ur);
                double pr = 0.01 * rho;
                Vw[q] = rho;
                Vw[nc + q] = amp * uvr;
                Vw[2 * nc + q] = 1.0 + amp * uvp;
                Vw[3 * nc + q] = amp * uvz;
                Vw[4 * nc + q] = 0.0;
                Vw[5 * nc + q] = sqrt(2.0 * pr / beta);
                Vw[6 * nc + q] = 0.0;
                Vw[7 * nc + q] = pr;
                Vw[8 * nc + q] = 0.0;
            }
    if (U || Uinit || rhofloor) {
        double *Uw = U ? U : Uinit ? Uinit : (double *)malloc(9 * nc * sizeof(double));
        if (!Uw) { if (!V) free(Vw); return MHD_ERR_NOMEM; }
        mhd_vtou(g, Vw, Uw);
        if (Uinit && Uinit != Uw) memcpy(Uinit, Uw, 9 * nc * sizeof(double));
        if (rhofloor)
            for (size_t q = 0; q < nc; q++) rhofloor[q] = Uw[q] * rhocr;
        if (!U && !Uinit) free(Uw);
    }
    if (Vinit) memcpy(Vinit, Vw, 9 * nc * sizeof(double));
    if (!V) free(Vw);
    return MHD_OK;
}

/* GalacticDisc3() (model.h:149-327): isothermal exponential gas disc
 * (exp(-R/rdisc) in the midplane, hydrostatic in z) plus a hydrostatic
 * isothermal halo in the fixed potential, rotation from radial balance in
 * the frame rotating at omegasp, toroidal field of plasma beta 1e4 at R=0.
 * Then VtoU, the z=0 symmetry fills of U (ZLeftVzAntisymBSymBoundary then
 * ZLeftFreeBoundary, zboundary.h:67-96,170-190) and SaveInitial.  The
 * reference evaluates the potentials in an OpenMP region, so the constant
 * terms are computed at run time here too (through volatile reads) rather
 * than folded by the compiler. */
int mhd_ic_galactic_disc3(const mhd_grid *g, const mhd_params *p, double *U, double *V, double *Uinit,
                          double *Vinit, double *rhofloor)
{
    if (!g || !p || !U || !V) return MHD_ERR_ARG;
    const size_t ixmax = (size_t)g->ix + 2, jymax = (size_t)g->jy + 2, kzmax = (size_t)g->kz + 2;
    const size_t nc = ixmax * jymax * kzmax;
    /* constant.h:48-84 */
    const double kpc = 3.08568e+21, mp = 1.673e-24, msun = 1.989e+33, v0 = 6.558e+6;
    const double l0 = (10 * kpc);
    volatile double pi4_v = 4.0 * M_PI;
    const double pi4 = pi4_v;
    volatile double knobs[7] = {GV_VHALO0, GV_DH, GV_A, GV_B, GV_MD, GV_DB, GV_MB};
    const double vhalo0 = knobs[0], dh = knobs[1], a = knobs[2], b = knobs[3], md = knobs[4], db = knobs[5],
                 mb = knobs[6];
    /* model.h:179-201 */
    const double mdisc = 0.4 * 0.75;
    const double rdisc = 0.7, zdisc = 0.03;
    const double discrho0 = (1.0e+10 * msun / (mp * 1000 * kpc * kpc * kpc) * mdisc / (pi4 * rdisc * rdisc * zdisc));
    const double csdisc2 = 1.33e+8 * 1.0e+4 / (v0 * v0);
    const double discbeta = 1.0e+4;
    const double halorho0 = 1.0e-4 * (1.0e+10 * msun / (mp * 1000 * kpc * kpc * kpc) * mdisc
                                      / (pi4 * rdisc * rdisc * zdisc));
    const double cshalo2 = 1.33e+8 * 2.4e+6 / (v0 * v0);
    const double oneocshalo2 = 1.0 / cshalo2;
    const double oneocsdisc2 = 1.0 / csdisc2;
    const double discbphi0 = sqrt(2.0 * csdisc2 * discrho0 / discbeta);
    const double omegasp = p->omegasp;
    for (size_t i = 0; i < ixmax; i++) {
        const double xi = g->x[i];
        for (size_t j = 0; j < jymax; j++)
            for (size_t k = 0; k < kzmax; k++) {
                const size_t q = (i * jymax + j) * kzmax + k;
                const double zk = g->z[k];
                const double x2 = xi * xi, z2 = zk * zk;
                /* model.h:214-227 */
                double potaxi = ((vhalo0 * vhalo0 * (2.0 * log(l0) + log(x2 + z2 + dh * dh)))
                                 - md / sqrt(x2 + (a + sqrt(z2 + b * b)) * (a + sqrt(z2 + b * b)))
                                 - mb / (sqrt(x2 + z2) + db));
                double potaxir = ((vhalo0 * vhalo0 * (2.0 * log(l0) + log(x2 + dh * dh)))
                                  - md / sqrt(x2 + (a + b) * (a + b))
                                  - mb / (xi + db));
                double potaxi0 = ((vhalo0 * vhalo0 * (2.0 * log(l0) + log(dh * dh)))
                                  - md / (a + b)
                                  - mb / db);
                double grx = axi_grx(xi, zk);
                /* model.h:251-293 */
                double halorho = halorho0 * exp(-oneocshalo2 * (potaxi - potaxi0));
                double halopr = cshalo2 * halorho;
                double discrho = (discrho0 * exp(-xi / rdisc) * exp(-oneocsdisc2 * (potaxi - potaxir)));
                double discpr = csdisc2 * discrho;
                double rho = discrho + halorho;
                V[q] = rho;
                V[nc + q] = 0.0;
                V[2 * nc + q] = (sqrt(-xi * (grx + csdisc2 / rdisc)) * discrho / rho - omegasp * xi);
                V[3 * nc + q] = 0.0;
                V[4 * nc + q] = 0.0;
                V[5 * nc + q] = (discbphi0 * exp(-xi / rdisc) / (cosh(zk / zdisc) * cosh(zk / zdisc)));
                V[6 * nc + q] = 0.0;
                V[7 * nc + q] = discpr + halopr;
                V[8 * nc + q] = 0.0;
            }
    }
    int rc = mhd_vtou(g, V, U);
    if (rc) return rc;
    /* zboundary.h:67-96 then :170-190 on U: k=0 <- k=2 (v_z odd), U3 at k=1 = 0,
     * then k=0 <- k=1 */
    for (size_t i = 0; i < ixmax; i++)
        for (size_t j = 0; j < jymax; j++) {
            const size_t q0 = (i * jymax + j) * kzmax;
            for (int m = 0; m < 9; m++)
                U[m * nc + q0] = (m == 3) ? -U[m * nc + q0 + 2] : U[m * nc + q0 + 2];
            U[3 * nc + q0 + 1] = 0.0;
            for (int m = 0; m < 9; m++) U[m * nc + q0] = U[m * nc + q0 + 1];
        }
    /* saveinitial.h:27-45 */
    if (Uinit) memcpy(Uinit, U, 9 * nc * sizeof(double));
    if (Vinit) memcpy(Vinit, V, 9 * nc * sizeof(double));
    if (rhofloor)
        for (size_t q = 0; q < nc; q++) rhofloor[q] = U[q] * p->rhocr;
    return MHD_OK;
}
