/*
 * mhd_oracle.c -- the ORACLE: CPU restatement of the reference's cylindrical
 * GLM-MHD TVD Runge-Kutta step.  Test infrastructure only (see mhd_oracle.h).
 *
 * Parity pinning: tests/test_oracle_ref.py runs this file against the
 * reference C compiled in place (oracle/_ref/, built by oracle/build_ref.py)
 * and requires bit-identical U, V, dt, ch and floor counters; committed golden
 * vectors made from the reference (tests/golden/) pin it on machines where the
 * reference tree is absent.
 *
 * Build with -O2 -ffp-contract=off (no fused multiply-add), like the reference
 * build, so every expression rounds exactly as the reference's does.  Every
 * expression below keeps the reference's evaluation order; parentheses added
 * here only spell out C's left-to-right grouping.
 *
 * Direction convention for the per-direction routines: dir 0 = r (x), 1 = phi
 * (y), 2 = z.  Normal velocity index n = 1+dir, normal field index bn = 4+dir,
 * tangential indices cyclic (t1 = 1+(dir+1)%3, t2 = 1+(dir+2)%3); the
 * reference's three per-direction files follow that cyclic order in every
 * tangential expression (e.g. hlldy.h:294 "sm*byint+vzll*bzll+vxll*bxll").
 */
#define _GNU_SOURCE
#include "mhd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* constant.h:62-79 */
static const double GM = 5.0 / 3.0;
static const double GM1 = 2.0 / 3.0;
static const double ONEOGM1 = 1.5;
static const double ONEOCR = 1.0 / 0.18;
static const double ONEO3 = 1.0 / 3.0;

struct orc_ctx {
    orc_gridspec gs;
    orc_params p;
    int ix, jy, kz, ixmax, jymax, kzmax, irin;
    size_t nc;                       /* cells per variable */
    double *x, *xm, *dx, *dxm, *oneox, *oneoxm, *oneodx, *y, *z, *zm, *dz, *dzm, *oneodz;
    double dy, oneody, minminlength, oneominminlength;
    double *g;                       /* [6][ixmax][kzmax]: g1..g6 (j-independent) */
    double *minlength;               /* [ixmax][kzmax] (j-independent) */
    double xabs[11], zabs[11], *cabs;/* cabs [irin+1][kzmax] */
    int *krin;
    double *U, *U1, *V, *S, *F, *G, *H, *Vl, *Vr;
    double *Uinit, *Vinit, *rhofloor;
    double *graxi, *gr;              /* [3][cells] */
    double dt, ch, t, psicoef;
    int counters[3];
};

#define IDX(o, i, j, k) ((((size_t)(i)) * (o)->jymax + (size_t)(j)) * (o)->kzmax + (size_t)(k))
#define A4(o, arr, m, i, j, k) (arr)[(size_t)(m) * (o)->nc + IDX(o, i, j, k)]

/* maxmin.h:16-26 */
static inline double rmax(double a, double b) { return a > b ? a : b; }
static inline double rmin(double a, double b) { return a > b ? b : a; }

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* grid: cylindricalgrid.h:25-227                                            */
/* ------------------------------------------------------------------------ */
static void build_grid(orc_ctx *o)
{
    const orc_gridspec *s = &o->gs;
    int ixmax1 = o->ixmax - 1, kzmax1 = o->kzmax - 1, jymax1 = o->jymax - 1;
    int i, j, k;

    o->dx[0] = s->dx0;
    o->x[0] = s->x0 - s->dx0;
    for (i = 0; i < ixmax1; i++) {
        o->x[i + 1] = o->x[i] + o->dx[i];
        if (o->x[i] > s->lx) o->dx[i + 1] = rmin(s->stretchratio * o->dx[i], s->dxmax);
        else o->dx[i + 1] = o->dx[i];
        o->xm[i] = (o->x[i] + o->x[i + 1]) * 0.5;
        o->dxm[i] = (o->dx[i] + o->dx[i + 1]) * 0.5;
        o->oneox[i] = 1.0 / o->x[i];
        o->oneoxm[i] = 1.0 / o->xm[i];
        o->oneodx[i] = 1.0 / o->dx[i];
    }
    o->xm[ixmax1] = o->x[ixmax1] + 0.5 * o->dx[ixmax1];
    o->dxm[ixmax1] = o->dx[ixmax1];
    o->oneox[ixmax1] = 1.0 / o->x[ixmax1];
    o->oneodx[ixmax1] = 1.0 / o->dx[ixmax1];

    o->dy = s->ly / (double)o->jy;
    o->y[0] = s->y0 - o->dy;
    o->oneody = 1.0 / o->dy;
    for (j = 0; j < jymax1; j++) o->y[j + 1] = o->y[j] + o->dy;

    o->dz[0] = s->dz0;
    o->z[0] = s->z0 - s->dz0;
    for (k = 0; k < kzmax1; k++) {
        o->z[k + 1] = o->z[k] + o->dz[k];
        if (o->z[k] > s->lz) o->dz[k + 1] = rmin(s->stretchratio * o->dz[k], s->dzmax);
        else o->dz[k + 1] = o->dz[k];
        o->zm[k] = (o->z[k] + o->z[k + 1]) * 0.5;
        o->dzm[k] = (o->dz[k] + o->dz[k + 1]) * 0.5;
        o->oneodz[k] = 1.0 / o->dz[k];
    }
    o->zm[kzmax1] = o->z[kzmax1] + 0.5 * o->dz[kzmax1];
    o->oneodz[kzmax1] = 1.0 / o->dz[kzmax1];

    /* cylindricalgrid.h:108-130: volume and face factors (j-independent) */
    for (i = 1; i < ixmax1; i++) {
        for (k = 1; k < kzmax1; k++) {
            double dvolume = 0.5 * (o->xm[i] * o->xm[i] - o->xm[i - 1] * o->xm[i - 1]) * o->dy * o->dzm[k - 1];
            double oneodvol = 1.0 / dvolume;
            size_t q = (size_t)i * o->kzmax + k, pl = (size_t)o->ixmax * o->kzmax;
            o->g[0 * pl + q] = o->xm[i - 1] * o->dy * o->dzm[k - 1] * oneodvol;
            o->g[1 * pl + q] = o->xm[i] * o->dy * o->dzm[k - 1] * oneodvol;
            o->g[2 * pl + q] = o->dxm[i - 1] * o->dzm[k - 1] * oneodvol;
            o->g[3 * pl + q] = o->g[2 * pl + q];
            o->g[4 * pl + q] = 0.5 * (o->xm[i] * o->xm[i] - o->xm[i - 1] * o->xm[i - 1]) * o->dy * oneodvol;
            o->g[5 * pl + q] = o->g[4 * pl + q];
        }
    }

    /* cylindricalgrid.h:136-163 */
    o->oneominminlength = 0.0;
    for (i = 0; i < o->ixmax; i++) {
        for (k = 0; k < o->kzmax; k++) {
            double ml = rmin(o->dx[i], rmin(o->x[i] * o->dy, o->dz[k]));
            double inv = 1.0 / ml;
            o->minlength[(size_t)i * o->kzmax + k] = ml;
            if (inv > o->oneominminlength) o->oneominminlength = inv;
        }
    }
    o->minminlength = 1.0 / o->oneominminlength;

    /* cylindricalgrid.h:168-201 */
    for (i = ixmax1 - 10; i < o->ixmax; i++)
        o->xabs[i - (ixmax1 - 10)] = (0.5 * (1.0 - tanh((o->x[ixmax1] - o->x[i] - 5.0 * o->dx[ixmax1])
                                                         / (2.0 * o->dx[ixmax1]))));
    for (k = kzmax1 - 10; k < o->kzmax; k++)
        o->zabs[k - (kzmax1 - 10)] = (0.5 * (1.0 - tanh((o->z[kzmax1] - o->z[k] - 5.0 * o->dz[kzmax1])
                                                         / (2.0 * o->dz[kzmax1]))));
    for (i = 0; i < o->irin + 1; i++) {
        for (k = 0; k < o->kzmax; k++) {
            double r = sqrt(o->x[i] * o->x[i] + o->z[k] * o->z[k]);
            o->cabs[(size_t)i * o->kzmax + k] = (0.5 * (1.0 - tanh((r - s->rin + 5.0 * s->dx0) / (2.0 * s->dx0))));
        }
    }
    /* cylindricalgrid.h:205-222 */
    for (i = 0; i < o->irin + 1; i++) {
        o->krin[i] = 0;
        for (k = 0; k < o->kzmax; k++) {
            double r = sqrt(o->x[i] * o->x[i] + o->z[k] * o->z[k]);
            if (r > s->rin) { o->krin[i] = k; break; }
        }
    }
}

orc_ctx *orc_create(const orc_gridspec *gs, const orc_params *p)
{
    orc_ctx *o = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    if (!o) return NULL;
    o->gs = *gs;
    o->p = *p;
    o->ix = gs->nr; o->jy = gs->nphi; o->kz = gs->nz;
    o->ixmax = o->ix + 2; o->jymax = o->jy + 2; o->kzmax = o->kz + 2;
    o->irin = (int)(gs->rin / gs->dx0);
    o->nc = (size_t)o->ixmax * o->jymax * o->kzmax;
#define ALLOC(ptr, n) do { (ptr) = (double *)calloc((n), sizeof(double)); if (!(ptr)) { orc_destroy(o); return NULL; } } while (0)
    ALLOC(o->x, o->ixmax); ALLOC(o->xm, o->ixmax); ALLOC(o->dx, o->ixmax); ALLOC(o->dxm, o->ixmax);
    ALLOC(o->oneox, o->ixmax); ALLOC(o->oneoxm, o->ixmax); ALLOC(o->oneodx, o->ixmax);
    ALLOC(o->y, o->jymax);
    ALLOC(o->z, o->kzmax); ALLOC(o->zm, o->kzmax); ALLOC(o->dz, o->kzmax); ALLOC(o->dzm, o->kzmax);
    ALLOC(o->oneodz, o->kzmax);
    ALLOC(o->g, 6 * (size_t)o->ixmax * o->kzmax);
    ALLOC(o->minlength, (size_t)o->ixmax * o->kzmax);
    ALLOC(o->cabs, (size_t)(o->irin + 1) * o->kzmax);
    o->krin = (int *)calloc((size_t)o->irin + 1, sizeof(int));
    ALLOC(o->U, 9 * o->nc); ALLOC(o->U1, 9 * o->nc); ALLOC(o->V, 9 * o->nc); ALLOC(o->S, 9 * o->nc);
    ALLOC(o->F, 9 * o->nc); ALLOC(o->G, 9 * o->nc); ALLOC(o->H, 9 * o->nc);
    ALLOC(o->Vl, 9 * o->nc); ALLOC(o->Vr, 9 * o->nc);
    ALLOC(o->Uinit, 9 * o->nc); ALLOC(o->Vinit, 9 * o->nc); ALLOC(o->rhofloor, o->nc);
    ALLOC(o->graxi, 3 * o->nc); ALLOC(o->gr, 3 * o->nc);
#undef ALLOC
    if (!o->krin) { orc_destroy(o); return NULL; }
    build_grid(o);
    return o;
}

void orc_destroy(orc_ctx *o)
{
    if (!o) return;
    double *bufs[] = {o->x, o->xm, o->dx, o->dxm, o->oneox, o->oneoxm, o->oneodx, o->y, o->z, o->zm,
                      o->dz, o->dzm, o->oneodz, o->g, o->minlength, o->cabs, o->U, o->U1, o->V, o->S,
                      o->F, o->G, o->H, o->Vl, o->Vr, o->Uinit, o->Vinit, o->rhofloor, o->graxi, o->gr};
    for (size_t q = 0; q < sizeof bufs / sizeof bufs[0]; q++) free(bufs[q]);
    free(o->krin);
    free(o);
}

void orc_dims(const orc_ctx *o, int *out)
{
    out[0] = o->ix; out[1] = o->jy; out[2] = o->kz;
    out[3] = o->ixmax; out[4] = o->jymax; out[5] = o->kzmax; out[6] = o->irin;
}

void orc_get_grid1d(const orc_ctx *o, double *x, double *xm, double *dx, double *dxm,
                    double *oneox, double *oneoxm, double *oneodx, double *y, double *z,
                    double *zm, double *dz, double *dzm, double *oneodz, double *scalars)
{
    size_t nx = (size_t)o->ixmax * sizeof(double), nz = (size_t)o->kzmax * sizeof(double);
    memcpy(x, o->x, nx); memcpy(xm, o->xm, nx); memcpy(dx, o->dx, nx); memcpy(dxm, o->dxm, nx);
    memcpy(oneox, o->oneox, nx); memcpy(oneoxm, o->oneoxm, nx - sizeof(double));
    memcpy(oneodx, o->oneodx, nx);
    memcpy(y, o->y, (size_t)o->jymax * sizeof(double));
    memcpy(z, o->z, nz); memcpy(zm, o->zm, nz); memcpy(dz, o->dz, nz); memcpy(dzm, o->dzm, nz);
    memcpy(oneodz, o->oneodz, nz);
    scalars[0] = o->dy; scalars[1] = o->oneody; scalars[2] = o->minminlength;
    scalars[3] = o->oneominminlength;
}

void orc_get_metric(const orc_ctx *o, double *g, double *minlen, double *xabs,
                    double *zabs, double *cabs, int *krin)
{
    int i, j, k, n;
    int a = o->ixmax - 1, b = o->jymax - 1, c = o->kzmax - 1;
    size_t pl = (size_t)o->ixmax * o->kzmax;
    for (n = 0; n < 6; n++)
        for (i = 0; i < a; i++)
            for (j = 0; j < b; j++)
                for (k = 0; k < c; k++) {
                    double v = 0.0;
                    if (i >= 1 && j >= 1 && k >= 1) v = o->g[n * pl + (size_t)i * o->kzmax + k];
                    g[(((size_t)n * a + i) * b + j) * c + k] = v;
                }
    for (i = 0; i < o->ixmax; i++)
        for (j = 0; j < o->jymax; j++)
            for (k = 0; k < o->kzmax; k++)
                minlen[IDX(o, i, j, k)] = o->minlength[(size_t)i * o->kzmax + k];
    memcpy(xabs, o->xabs, sizeof o->xabs);
    memcpy(zabs, o->zabs, sizeof o->zabs);
    memcpy(cabs, o->cabs, (size_t)(o->irin + 1) * o->kzmax * sizeof(double));
    memcpy(krin, o->krin, (size_t)(o->irin + 1) * sizeof(int));
}

/* ------------------------------------------------------------------------ */
/* gravity                                                                   */
/* ------------------------------------------------------------------------ */

/* initialgravity.h:22-79 (v0 = 6.558e+6, constant.h:78) */
void orc_initial_gravity(orc_ctx *o)
{
    const double vhalo0 = 131.5e+5 / 6.558e+6, dh = 1.2;
    const double a = 0.65, b = 0.026, md = 10.0;
    const double db = 0.07, mb = 3.4;
    int i, j, k;
#pragma omp parallel for private(j, k)
    for (i = 0; i < o->ixmax; i++) {
        for (j = 0; j < o->jymax; j++) {
            for (k = 0; k < o->kzmax; k++) {
                double x2 = o->x[i] * o->x[i];
                double z2 = o->z[k] * o->z[k];
                size_t q = IDX(o, i, j, k);
                o->graxi[q] = ((-2.0 * vhalo0 * vhalo0 / (x2 + z2 + dh * dh)
                                - md / pow(x2 + (a + sqrt(z2 + b * b)) * (a + sqrt(z2 + b * b)), 1.5)
                                - mb / ((sqrt(x2 + z2) + db) * (sqrt(x2 + z2) + db) * sqrt(x2 + z2)))
                               * o->x[i]);
                o->graxi[o->nc + q] = 0.0;
                o->graxi[2 * o->nc + q] = ((-2.0 * vhalo0 * vhalo0 / (x2 + z2 + dh * dh)
                                            - md / pow(x2 + (a + sqrt(z2 + b * b)) * (a + sqrt(z2 + b * b)), 1.5)
                                              * (1.0 + a / sqrt(z2 + b * b))
                                            - mb / ((sqrt(x2 + z2) + db) * (sqrt(x2 + z2) + db) * sqrt(x2 + z2)))
                                           * o->z[k]);
            }
        }
    }
}

void orc_set_gravity_axi(orc_ctx *o, const double *axi)
{
    memcpy(o->graxi, axi, 3 * o->nc * sizeof(double));
}

void orc_get_gravity(const orc_ctx *o, double *axi, double *gr)
{
    if (axi) memcpy(axi, o->graxi, 3 * o->nc * sizeof(double));
    if (gr) memcpy(gr, o->gr, 3 * o->nc * sizeof(double));
}

/* spiralgravity.h:20-124 (m[1]=10, a[1]=0.65, b[1]=0.026; cot(p)=1/tan(p)) */
void orc_spiral_gravity(orc_ctx *o, double t)
{
    const orc_params *p = &o->p;
    const double m1 = 10.0, a1 = 0.65, b1 = 0.026;
    double oneoscalephase = 1.0 / p->scalephase;
    double oneoscaler = 1.0 / p->scaler;
    double cotpitch = 1.0 / tan(p->pitch);
    double switchfunc = (t - p->tausp) / fabs(t - p->tausp);
    double epssp = 0.5 * p->epssp0 * (t / p->tausp * (1.0 - switchfunc) + (1.0 + switchfunc));
    double armnum = (double)(int)p->armnum;
    int i;
    o->t = t;
#pragma omp parallel for
    for (i = 0; i < o->ixmax; i++) {
        double xi = o->x[i];
        double x2 = xi * xi;
        double xoscalephase = xi * oneoscalephase;
        double xoscaler = xi * oneoscaler;
        double xoscaler2 = xoscaler * oneoscaler;
        double x2oscaler2 = xoscaler * xoscaler;
        double oneoonex2oscaler2 = 1.0 / (1.0 + x2oscaler2);
        double oneoonex2oscaler215 = 1.0 * pow(oneoonex2oscaler2, 1.5);
        double xoscaler2oonex2oscaler215 = xoscaler2 * oneoonex2oscaler215;
        double x2oscaler2oonex2oscaler215 = x2oscaler2 * oneoonex2oscaler215;
        for (int j = 0; j < o->jymax; j++) {
            double phase = armnum * (o->y[j] - (p->omegapattern - p->omegasp) * t
                                     + cotpitch * log(xoscalephase));
            double sinphase, cosphase;
            sincos(phase, &sinphase, &cosphase);
            for (int k = 0; k < o->kzmax; k++) {
                double zk = o->z[k];
                double z2 = zk * zk;
                double a1zk2b12 = ((a1 + sqrt(z2 + b1 * b1)) * (a1 + sqrt(z2 + b1 * b1)));
                double oneosqrtx2a1zk2b12 = 1.0 / sqrt(x2 + a1zk2b12);
                double scalezosqrtz2scalez2 = (p->scalez / sqrt(z2 + p->scalez * p->scalez));
                double spiralfr = (-epssp * m1 * oneosqrtx2a1zk2b12 * scalezosqrtz2scalez2
                                   * xoscaler2oonex2oscaler215
                                   * ((xi * oneosqrtx2a1zk2b12 * oneosqrtx2a1zk2b12
                                       - ((2.0 - x2oscaler2) * oneoonex2oscaler2)) * cosphase
                                      + armnum * cotpitch * sinphase));
                double spiralfphi = (epssp * m1 * oneosqrtx2a1zk2b12 * scalezosqrtz2scalez2
                                     * xoscaler2oonex2oscaler215 * armnum * sinphase);
                double spiralfz = (-epssp * m1 * oneosqrtx2a1zk2b12 * zk * scalezosqrtz2scalez2
                                   * x2oscaler2oonex2oscaler215
                                   * ((1.0 + a1 / sqrt(z2 + b1 * b1)) * oneosqrtx2a1zk2b12 * oneosqrtx2a1zk2b12
                                      + 1.0 / (z2 + p->scalez * p->scalez)) * cosphase);
                size_t q = IDX(o, i, j, k);
                o->gr[q] = o->graxi[q] + spiralfr;
                o->gr[o->nc + q] = o->graxi[o->nc + q] + spiralfphi;
                o->gr[2 * o->nc + q] = o->graxi[2 * o->nc + q] + spiralfz;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* state I/O                                                                 */
/* ------------------------------------------------------------------------ */
void orc_load(orc_ctx *o, const double *U, const double *V, const double *Uinit,
              const double *Vinit, const double *rhofloor)
{
    size_t n9 = 9 * o->nc * sizeof(double);
    memcpy(o->U, U, n9); memcpy(o->V, V, n9);
    memcpy(o->Uinit, Uinit, n9); memcpy(o->Vinit, Vinit, n9);
    memcpy(o->rhofloor, rhofloor, o->nc * sizeof(double));
}

/* The benchmark's seeded disc, generated in place so a full-size CPU run needs
 * no second copy of the state: rho = exp(-z^2/(2*0.1^2)) + 1e-3, p = 0.01 rho,
 * v_phi = 1, B_phi = sqrt(2p/beta), with uniform [-1,1) perturbations of
 * relative size amp on rho and of size amp on v (four splitmix64 draws per
 * cell, cells in [i][j][k] order, ghosts included).  Then VtoU (vtou.h:20-62)
 * and SaveInitial's copies and density floor (saveinitial.h:30-41). */
static unsigned long long orc_splitmix64(unsigned long long *s)
{
    unsigned long long z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double orc_unit_pm(unsigned long long *s)
{
    return 2.0 * ((double)(orc_splitmix64(s) >> 11) * 0x1.0p-53) - 1.0;
}

void orc_ic_disc(orc_ctx *o, double beta, double amp, unsigned long long seed)
{
    const size_t nc = o->nc;
    unsigned long long st = seed;
    size_t q = 0;
    for (int i = 0; i < o->ixmax; i++)
        for (int j = 0; j < o->jymax; j++)
            for (int k = 0; k < o->kzmax; k++, q++) {
                double zk = o->z[k];
                double rho = exp(-zk * zk / (2.0 * 0.1 * 0.1)) + 1.0e-3;
                double ur = orc_unit_pm(&st), uvr = orc_unit_pm(&st), uvp = orc_unit_pm(&st), uvz = orc_unit_pm(&st);
                rho = rho * (1.0 + amp * ur);
                double pr = 0.01 * rho;
                double *v = o->V;
                v[q] = rho;
                v[nc + q] = amp * uvr;
                v[2 * nc + q] = 1.0 + amp * uvp;
                v[3 * nc + q] = amp * uvz;
                v[4 * nc + q] = 0.0;
                v[5 * nc + q] = sqrt(2.0 * pr / beta);
                v[6 * nc + q] = 0.0;
                v[7 * nc + q] = pr;
                v[8 * nc + q] = 0.0;
            }
#pragma omp parallel for
    for (int i = 0; i < o->ixmax; i++) {
        const double xi = o->x[i];
        for (size_t c = (size_t)i * o->jymax * o->kzmax; c < (size_t)(i + 1) * o->jymax * o->kzmax; c++) {
            const double *v = o->V;
            double *u = o->U;
            double v2 = v[nc + c] * v[nc + c] + v[2 * nc + c] * v[2 * nc + c] + v[3 * nc + c] * v[3 * nc + c];
            double b2 = v[4 * nc + c] * v[4 * nc + c] + v[5 * nc + c] * v[5 * nc + c] + v[6 * nc + c] * v[6 * nc + c];
            u[c] = v[c];
            u[nc + c] = v[c] * v[nc + c];
            u[2 * nc + c] = xi * v[c] * v[2 * nc + c];
            u[3 * nc + c] = v[c] * v[3 * nc + c];
            u[4 * nc + c] = v[4 * nc + c];
            u[5 * nc + c] = v[5 * nc + c];
            u[6 * nc + c] = v[6 * nc + c];
            u[7 * nc + c] = 0.5 * (v[c] * v2 + b2) + ONEOGM1 * v[7 * nc + c];
            u[8 * nc + c] = v[8 * nc + c];
            for (int m = 0; m < 9; m++) {
                o->Uinit[m * nc + c] = u[m * nc + c];
                o->Vinit[m * nc + c] = v[m * nc + c];
            }
            o->rhofloor[c] = u[c] * o->p.rhocr;
        }
    }
}

void orc_store(const orc_ctx *o, double *U, double *V, double *U1)
{
    size_t n9 = 9 * o->nc * sizeof(double);
    if (U) memcpy(U, o->U, n9);
    if (V) memcpy(V, o->V, n9);
    if (U1) memcpy(U1, o->U1, n9);
}

/* ------------------------------------------------------------------------ */
/* cooling.h:22-78 (a=0.031, b=0.054, c=0.078, d=0.235; B=C=0)               */
/* te0 = mu*mp/kb*v0*v0 as constant.h:81 spells it                          */
/* ------------------------------------------------------------------------ */
int orc_cooling(double rho, double pr)
{
    const double te0 = ((0.619047619 * 1.673e-24) * (1.0 / 1.3806504e-16) * 6.558e+6 * 6.558e+6);
    double temperature = pr / rho;
    double a = 0.031, b = 0.054, c = 0.078, d = 0.235;
    double tempma = temperature - a, fabstempma = fabs(tempma);
    double tempmb = temperature - b, fabstempmb = fabs(tempmb);
    double tempmc = temperature - c, fabstempmc = fabs(tempmc);
    double tempmd = temperature - d, fabstempmd = fabs(tempmd);
    double signa = tempma / fabstempma;
    double signb = tempmb / fabstempmb;
    double signc = tempmc / fabstempmc;
    double signd = tempmd / fabstempmd;
    double A = 0.108e-37 * pow(te0 * temperature, 10.26);
    double B = 0.0, C = 0.0;
    return (0.5 * (A * (1.0 - signa * signb) + B * (1.0 - signb * signc) + C * (1.0 - signc * signd)));
}

static inline int cool(const orc_ctx *o, double rho, double pr)
{
    return o->p.cooling ? orc_cooling(rho, pr) : 0;
}

/* ------------------------------------------------------------------------ */
/* setdt.h:24-94 (serial semantics: first cell reaching the strict maximum)  */
/* ------------------------------------------------------------------------ */
void orc_setdt(orc_ctx *o, double *dt, double *ch, int *ijk)
{
    double best = 0.0;
    long bestq = -1;
    int i;
    const double *V = o->V;
#pragma omp parallel
    {
        double lbest = 0.0;
        long lq = -1;
#pragma omp for schedule(static) nowait
        for (i = 1; i < o->ixmax - 1 - 10; i++) {
            for (int j = 1; j < o->jymax - 1; j++) {
                for (int k = 1; k < o->kzmax - 1; k++) {
                    size_t q = IDX(o, i, j, k);
                    double v0 = V[q], v1 = V[o->nc + q], v2v = V[2 * o->nc + q], v3 = V[3 * o->nc + q];
                    double v4 = V[4 * o->nc + q], v5 = V[5 * o->nc + q], v6 = V[6 * o->nc + q];
                    double v7 = V[7 * o->nc + q];
                    double v2 = v1 * v1 + v2v * v2v + v3 * v3;
                    double b2 = v4 * v4 + v5 * v5 + v6 * v6;
                    double t1 = sqrt(v2 + (GM * v7 + b2) / v0) / o->minlength[(size_t)i * o->kzmax + k];
                    double tc = (2.0 * ((v0 * v0 * cool(o, v0, v7)) / (1.5 * v7)));
                    double tmp = rmax(t1, tc);
                    if (tmp > lbest) { lbest = tmp; lq = (long)q; }
                }
            }
        }
#pragma omp critical
        {
            if (lq >= 0 && (lbest > best || (lbest == best && (bestq < 0 || lq < bestq)))) {
                best = lbest; bestq = lq;
            }
        }
    }
    o->dt = o->p.cfl / best;
    o->ch = o->minminlength * best;
    *dt = o->dt; *ch = o->ch;
    if (ijk) {
        if (bestq < 0) { ijk[0] = ijk[1] = ijk[2] = -1; }
        else {
            ijk[2] = (int)(bestq % o->kzmax);
            ijk[1] = (int)((bestq / o->kzmax) % o->jymax);
            ijk[0] = (int)(bestq / ((long)o->kzmax * o->jymax));
        }
    }
}

/* ------------------------------------------------------------------------ */
/* glmsourcesolver.h:19-47                                                   */
/* ------------------------------------------------------------------------ */
static void glm_damp(orc_ctx *o, double *Ud)
{
    double *u8 = Ud + 8 * o->nc, *v8 = o->V + 8 * o->nc;
    size_t q;
#pragma omp parallel for
    for (q = 0; q < o->nc; q++) {
        u8[q] = o->psicoef * u8[q];
        v8[q] = o->psicoef * v8[q];
    }
}

/* ------------------------------------------------------------------------ */
/* limiters                                                                  */
/* ------------------------------------------------------------------------ */

/* fast magnetosonic speed with normal field bnv (limiterx.h:189-198) */
static inline double fast_speed(double v0, double v4, double v5, double v6, double v7, double bnv)
{
    double b2 = (v4 * v4 + v5 * v5 + v6 * v6);
    double gmpr = GM * v7;
    return sqrt(((b2 + gmpr) + sqrt((b2 + gmpr) * (b2 + gmpr) - 4.0 * gmpr * bnv * bnv)) / (2.0 * v0));
}

/* minmod with characteristic correction: limiterx.h:171-217 (dir 0),
 * limitery.h:46-94 (dir 1), limiterz.h:146-190 (dir 2) */
static void minmod_limiter(orc_ctx *o, int dir)
{
    const double *V = o->V;
    double *Vl = o->Vl, *Vr = o->Vr;
    int ilo = dir == 0 ? 1 : 0, jlo = dir == 1 ? 1 : 0, klo = dir == 2 ? 1 : 0;
    int ihi = o->ixmax - 1, jhi = o->jymax - 1, khi = o->kzmax - 1;
    size_t st = dir == 0 ? (size_t)o->jymax * o->kzmax : dir == 1 ? (size_t)o->kzmax : 1;
    int n = 1 + dir, bn = 4 + dir;
    double dt = o->dt;
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++) {
        for (int i = ilo; i < ihi; i++) {
            for (int j = jlo; j < jhi; j++) {
                for (int k = klo; k < khi; k++) {
                    size_t q = IDX(o, i, j, k);
                    const double *vm = V + (size_t)m * o->nc;
                    double a = vm[q] - vm[q - st];
                    double b = vm[q + st] - vm[q];
                    double grad;
                    if (a * b <= 0.0) grad = 0.0;
                    else {
                        if (a > 0.0) grad = rmin(a, b);
                        else grad = rmax(a, b);
                    }
                    double fast = fast_speed(V[q], V[4 * o->nc + q], V[5 * o->nc + q], V[6 * o->nc + q],
                                             V[7 * o->nc + q], V[(size_t)bn * o->nc + q]);
                    double vn = V[(size_t)n * o->nc + q];
                    double lambmax = rmax(0.0, vn + fast);
                    double lambmin = rmin(0.0, vn - fast);
                    double *vl = Vl + (size_t)m * o->nc, *vr = Vr + (size_t)m * o->nc;
                    if (dir == 0) {
                        vl[q] = (vm[q] + 0.5 * (1.0 - lambmax * dt * o->oneodx[i]) * grad);
                        vr[q - st] = (vm[q] - 0.5 * (1.0 + lambmin * dt * o->oneodx[i - 1]) * grad);
                    } else if (dir == 1) {
                        vl[q] = (vm[q] + 0.5 * (1.0 - lambmax * dt * o->oneox[i] * o->oneody) * grad);
                        vr[q - st] = (vm[q] - 0.5 * (1.0 + lambmin * dt * o->oneox[i] * o->oneody) * grad);
                    } else {
                        vl[q] = (vm[q] + 0.5 * (1.0 - lambmax * dt * o->oneodz[k]) * grad);
                        vr[q - st] = (vm[q] - 0.5 * (1.0 + lambmin * dt * o->oneodz[k - 1]) * grad);
                    }
                }
            }
        }
    }
}

/* MC: limiterx.h:346-373, limitery.h:208-235, limiterz.h:305-332 */
static void mc_limiter(orc_ctx *o, int dir)
{
    const double *V = o->V;
    int ilo = dir == 0 ? 1 : 0, jlo = dir == 1 ? 1 : 0, klo = dir == 2 ? 1 : 0;
    int ihi = o->ixmax - 1, jhi = o->jymax - 1, khi = o->kzmax - 1;
    size_t st = dir == 0 ? (size_t)o->jymax * o->kzmax : dir == 1 ? (size_t)o->kzmax : 1;
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++) {
        const double *vm = V + (size_t)m * o->nc;
        double *vl = o->Vl + (size_t)m * o->nc, *vr = o->Vr + (size_t)m * o->nc;
        for (int i = ilo; i < ihi; i++) {
            for (int j = jlo; j < jhi; j++) {
                for (int k = klo; k < khi; k++) {
                    size_t q = IDX(o, i, j, k);
                    double a = vm[q] - vm[q - st];
                    double b = vm[q + st] - vm[q];
                    double c = 0.25 * (vm[q + st] - vm[q - st]);
                    double grad;
                    if (a * b <= 0.0) grad = 0.0;
                    else {
                        if (a > 0.0) grad = rmin(a, rmin(b, c));
                        else grad = rmax(a, rmax(b, c));
                    }
                    vl[q] = vm[q] + grad;
                    vr[q - st] = vm[q] - grad;
                }
            }
        }
    }
}

/* van Leer (limiterx.h:266-326, limitery.h:129-188, limiterz.h:232-285) and
 * superbee (limiterx.h:394-449, limitery.h:256-311, limiterz.h:367-432) */
static void vl_sb_limiter(orc_ctx *o, int dir, int superbee)
{
    const double *V = o->V;
    int ilo = dir == 0 ? 1 : 0, jlo = dir == 1 ? 1 : 0, klo = dir == 2 ? 1 : 0;
    int ihi = o->ixmax - 1, jhi = o->jymax - 1, khi = o->kzmax - 1;
    size_t st = dir == 0 ? (size_t)o->jymax * o->kzmax : dir == 1 ? (size_t)o->kzmax : 1;
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++) {
        const double *vm = V + (size_t)m * o->nc;
        double *vl = o->Vl + (size_t)m * o->nc, *vr = o->Vr + (size_t)m * o->nc;
        for (int i = ilo; i < ihi; i++)
            for (int j = jlo; j < jhi; j++)
                for (int k = klo; k < khi; k++) {
                    size_t q = IDX(o, i, j, k);
                    double a = vm[q] - vm[q - st];
                    double b = vm[q + st] - vm[q];
                    double grad;
                    if (a * b <= 0.0) grad = 0.0;
                    else if (!superbee) grad = a * b / (a + b);
                    else if (fabs(a) >= fabs(b)) grad = (a > 0.0) ? rmin(a, 2.0 * b) : rmax(a, 2.0 * b);
                    else grad = (a > 0.0) ? rmin(2.0 * a, b) : rmax(2.0 * a, b);
                    if (superbee) grad = 0.5 * grad;
                    vl[q] = vm[q] + grad;
                    vr[q - st] = vm[q] - grad;
                }
    }
}

/* the free fill of one direction (xvlrboundary.h:189-214 and the y, z
 * analogues): Vl of the first face <- its Vr, Vr of the last face <- its Vl */
static void vlr_free(orc_ctx *o, int dir)
{
    int n[3] = {o->ixmax - 1, o->jymax - 1, o->kzmax - 1};
    int last = n[dir] - 1, m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < n[0]; i++)
            for (int j = 0; j < n[1]; j++)
                for (int k = 0; k < n[2]; k++) {
                    int c = dir == 0 ? i : dir == 1 ? j : k;
                    if (c == 0) A4(o, o->Vl, m, i, j, k) = A4(o, o->Vr, m, i, j, k);
                    if (c == last) A4(o, o->Vr, m, i, j, k) = A4(o, o->Vl, m, i, j, k);
                }
}

/* YVlrInitializeBoundary (yvlrboundary.h:26-52) */
static void vlr_initialize_y(orc_ctx *o)
{
    int ixmax1 = o->ixmax - 1, jymax1 = o->jymax - 1, kzmax1 = o->kzmax - 1, m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < ixmax1; i++)
            for (int k = 0; k < kzmax1; k++) {
                A4(o, o->Vl, m, i, 0, k) = A4(o, o->Vinit, m, i, 0, k);
                A4(o, o->Vr, m, i, jymax1 - 1, k) = A4(o, o->Vinit, m, i, jymax1, k);
            }
}

/* the periodic fill along z (zvlrboundary.h:101-126) */
static void vlr_periodic_z(orc_ctx *o)
{
    int ixmax1 = o->ixmax - 1, jymax1 = o->jymax - 1, kzmax1 = o->kzmax - 1, m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < ixmax1; i++)
            for (int j = 0; j < jymax1; j++) {
                A4(o, o->Vl, m, i, j, 0) = A4(o, o->Vl, m, i, j, kzmax1 - 1);
                A4(o, o->Vr, m, i, j, kzmax1 - 1) = A4(o, o->Vr, m, i, j, 0);
            }
}

/* left/right state boundaries applied inside the limiters:
 * x: XVlrPeriodicBoundary (xvlrboundary.h:153-180, limiterx.h:252,380)
 * y: YVlrPeriodicBoundary (yvlrboundary.h:61-87, limitery.h:108,242)
 * z minmod: ZLeftVlVzAntisymBzsymBoundary + ZRightVrFreeBoundary
 *           (zvlrboundary.h:63-92,28-54; limiterz.h:197,204)
 * z MC: ZVlrFixedBoundary (zvlrboundary.h:173-200; limiterz.h:353) */
static void vlr_boundary(orc_ctx *o, int dir)
{
    int ixmax1 = o->ixmax - 1, jymax1 = o->jymax - 1, kzmax1 = o->kzmax - 1;
    int m;
    if (dir == 0) {
#pragma omp parallel for
        for (m = 0; m < 9; m++)
            for (int j = 0; j < jymax1; j++)
                for (int k = 0; k < kzmax1; k++) {
                    A4(o, o->Vl, m, 0, j, k) = A4(o, o->Vl, m, ixmax1 - 1, j, k);
                    A4(o, o->Vr, m, ixmax1 - 1, j, k) = A4(o, o->Vr, m, 0, j, k);
                }
    } else if (dir == 1) {
#pragma omp parallel for
        for (m = 0; m < 9; m++)
            for (int i = 0; i < ixmax1; i++)
                for (int k = 0; k < kzmax1; k++) {
                    A4(o, o->Vl, m, i, 0, k) = A4(o, o->Vl, m, i, jymax1 - 1, k);
                    A4(o, o->Vr, m, i, jymax1 - 1, k) = A4(o, o->Vr, m, i, 0, k);
                }
    } else if (o->p.limiter == 0) {
        int i;
#pragma omp parallel for
        for (i = 0; i < ixmax1; i++)
            for (int j = 0; j < jymax1; j++)
                for (m = 0; m < 9; m++)
                    A4(o, o->Vl, m, i, j, 0) = (m == 3) ? -A4(o, o->Vr, m, i, j, 1) : A4(o, o->Vr, m, i, j, 1);
#pragma omp parallel for
        for (m = 0; m < 9; m++)
            for (int i2 = 0; i2 < ixmax1; i2++)
                for (int j = 0; j < jymax1; j++)
                    A4(o, o->Vr, m, i2, j, kzmax1 - 1) = A4(o, o->Vl, m, i2, j, kzmax1 - 1);
    } else {
#pragma omp parallel for
        for (m = 0; m < 9; m++)
            for (int i = 0; i < ixmax1; i++)
                for (int j = 0; j < jymax1; j++) {
                    A4(o, o->Vl, m, i, j, 0) = A4(o, o->Vinit, m, i, j, 0);
                    A4(o, o->Vr, m, i, j, kzmax1 - 1) = A4(o, o->Vinit, m, i, j, kzmax1);
                }
    }
}

static void limiter(orc_ctx *o, int dir)
{
    if (o->p.limiter == 2) {
        /* van Leer: free in x (limiterx.h:314), periodic then initialize in y
         * (limitery.h:176,183), free in z (limiterz.h:273) */
        vl_sb_limiter(o, dir, 0);
        if (dir == 1) { vlr_boundary(o, 1); vlr_initialize_y(o); }
        else vlr_free(o, dir);
        return;
    }
    if (o->p.limiter == 3) {
        /* superbee: periodic in x, y, z (limiterx.h:444, limitery.h:306, limiterz.h:419) */
        vl_sb_limiter(o, dir, 1);
        if (dir == 2) vlr_periodic_z(o);
        else vlr_boundary(o, dir);
        return;
    }
    if (o->p.limiter == 0) minmod_limiter(o, dir);
    else mc_limiter(o, dir);
    vlr_boundary(o, dir);
}

/* ------------------------------------------------------------------------ */
/* face conversions and Riemann solvers                                      */
/* ------------------------------------------------------------------------ */

/* vlrtoulr.h:25-43; r = xm[i] for the r sweep, x[i] for phi and z */
static inline void prim_to_cons(const double *W, double v2, double b2, double r, double *Uo)
{
    Uo[0] = W[0];
    Uo[1] = W[0] * W[1];
    Uo[2] = r * W[0] * W[2];
    Uo[3] = W[0] * W[3];
    Uo[4] = W[4];
    Uo[5] = W[5];
    Uo[6] = W[6];
    Uo[7] = 0.5 * (W[0] * v2 + b2) + ONEOGM1 * W[7];
    Uo[8] = W[8];
}

/* physical flux of one face state: vlrulrtoflr.h:24-51 (dir 0, r=xm[i]),
 * vlrulrtoglr.h:25-53 (dir 1, r=x[i], oneor=oneox[i]), vlrulrtohlr.h:24-52
 * (dir 2, r=x[i]) */
static inline void side_flux(int dir, const double *W, const double *Uw, double b2, double vdotb,
                             double r, double oneor, double *Fo)
{
    if (dir == 0) {
        Fo[0] = Uw[1];
        Fo[1] = Uw[1] * W[1] + (W[7] + 0.5 * b2) - W[4] * W[4];
        Fo[2] = Uw[2] * W[1] - r * W[5] * W[4];
        Fo[3] = Uw[3] * W[1] - W[6] * W[4];
        Fo[4] = 0.0;
        Fo[5] = W[5] * W[1] - W[2] * W[4];
        Fo[6] = W[6] * W[1] - W[3] * W[4];
        Fo[7] = (Uw[7] + W[7] + 0.5 * b2) * W[1] - vdotb * W[4];
    } else if (dir == 1) {
        Fo[0] = Uw[2] * oneor;
        Fo[1] = Uw[1] * W[2] - W[4] * W[5];
        Fo[2] = Uw[2] * W[2] + r * ((W[7] + 0.5 * b2) - W[5] * W[5]);
        Fo[3] = Uw[3] * W[2] - W[6] * W[5];
        Fo[4] = W[4] * W[2] - W[1] * W[5];
        Fo[5] = 0.0;
        Fo[6] = W[6] * W[2] - W[3] * W[5];
        Fo[7] = (Uw[7] + W[7] + 0.5 * b2) * W[2] - vdotb * W[5];
    } else {
        Fo[0] = Uw[3];
        Fo[1] = Uw[1] * W[3] - W[4] * W[6];
        Fo[2] = Uw[2] * W[3] - r * W[5] * W[6];
        Fo[3] = Uw[3] * W[3] + (W[7] + 0.5 * b2) - W[6] * W[6];
        Fo[4] = W[4] * W[3] - W[1] * W[6];
        Fo[5] = W[5] * W[3] - W[2] * W[6];
        Fo[6] = 0.0;
        Fo[7] = (Uw[7] + W[7] + 0.5 * b2) * W[3] - vdotb * W[6];
    }
}

/* flux of an intermediate (star) state given physical components v[1..3],
 * b[1..3]: primitivetof.h:22-41, primitivetog.h:22-41, primitivetoh.h:22-41 */
static inline void star_flux(int dir, double vdotb, double rho, const double *v, const double *b,
                             double en, double ptot, double r, double *Fo)
{
    double vx = v[1], vy = v[2], vz = v[3], bx = b[1], by = b[2], bz = b[3];
    if (dir == 0) {
        Fo[0] = rho * vx;
        Fo[1] = rho * vx * vx + ptot - bx * bx;
        Fo[2] = r * (rho * vy * vx - by * bx);
        Fo[3] = rho * vz * vx - bz * bx;
        Fo[4] = 0.0;
        Fo[5] = by * vx - vy * bx;
        Fo[6] = bz * vx - vz * bx;
        Fo[7] = (en + ptot) * vx - vdotb * bx;
    } else if (dir == 1) {
        Fo[0] = rho * vy;
        Fo[1] = rho * vx * vy - bx * by;
        Fo[2] = r * (rho * vy * vy + ptot - by * by);
        Fo[3] = rho * vz * vy - bz * by;
        Fo[4] = bx * vy - vx * by;
        Fo[5] = 0.0;
        Fo[6] = bz * vy - vz * by;
        Fo[7] = (en + ptot) * vy - vdotb * by;
    } else {
        Fo[0] = rho * vz;
        Fo[1] = rho * vx * vz - bx * bz;
        Fo[2] = r * (rho * vy * vz - by * bz);
        Fo[3] = rho * vz * vz + ptot - bz * bz;
        Fo[4] = bx * vz - vx * bz;
        Fo[5] = by * vz - vy * bz;
        Fo[6] = 0.0;
        Fo[7] = (en + ptot) * vz - vdotb * bz;
    }
}

/* HLLD (Miyoshi & Kusano 2005) as written in hlldx.h:58-471 (dir 0),
 * hlldy.h:60-479 (dir 1), hlldz.h:58-475 (dir 2) */
static void hlld_face(int dir, const double *L, const double *R, double r, double oneor, double *Fo)
{
    int n = 1 + dir, bn = 4 + dir;
    int t1 = 1 + (dir + 1) % 3, t2 = 1 + (dir + 2) % 3;
    int bt1 = t1 + 3, bt2 = t2 + 3;
    double Ul[9], Ur[9];

    double vl2 = L[1] * L[1] + L[2] * L[2] + L[3] * L[3];
    double bl2 = L[4] * L[4] + L[5] * L[5] + L[6] * L[6];
    double vldotbl = L[1] * L[4] + L[2] * L[5] + L[3] * L[6];
    double gmpr = GM * L[7];
    double ptl = L[7] + 0.5 * bl2;
    double vfl = sqrt(((bl2 + gmpr) + sqrt((bl2 + gmpr) * (bl2 + gmpr) - 4.0 * gmpr * L[bn] * L[bn])) / (2.0 * L[0]));

    double vr2 = R[1] * R[1] + R[2] * R[2] + R[3] * R[3];
    double br2 = R[4] * R[4] + R[5] * R[5] + R[6] * R[6];
    double vrdotbr = R[1] * R[4] + R[2] * R[5] + R[3] * R[6];
    gmpr = GM * R[7];
    double ptr = R[7] + 0.5 * br2;
    double vfr = sqrt(((br2 + gmpr) + sqrt((br2 + gmpr) * (br2 + gmpr) - 4.0 * gmpr * R[bn] * R[bn])) / (2.0 * R[0]));

    double sl = rmin(L[n], R[n]) - rmax(vfl, vfr);
    double sr = rmax(L[n], R[n]) + rmax(vfl, vfr);

    if (sl >= 0.0) {
        prim_to_cons(L, vl2, bl2, r, Ul);
        side_flux(dir, L, Ul, bl2, vldotbl, r, oneor, Fo);
        return;
    }
    if (sr <= 0.0) {
        prim_to_cons(R, vr2, br2, r, Ur);
        side_flux(dir, R, Ur, br2, vrdotbr, r, oneor, Fo);
        return;
    }
    prim_to_cons(L, vl2, bl2, r, Ul);
    prim_to_cons(R, vr2, br2, r, Ur);

    double slvl = sl - L[n];
    double srvr = sr - R[n];
    double sm;
    if (dir == 1)
        sm = ((srvr * R[0] * R[2] - slvl * L[0] * L[2]) - ptr + ptl) / (srvr * Ur[0] - slvl * Ul[0]);
    else
        sm = (srvr * Ur[n] - slvl * Ul[n] - ptr + ptl) / (srvr * Ur[0] - slvl * Ul[0]);
    double oneoslsm = 1.0 / (sl - sm);
    double oneosrsm = 1.0 / (sr - sm);
    double ptint = (srvr * Ur[0] * ptl - slvl * Ul[0] * ptr
                    + Ur[0] * Ul[0] * srvr * slvl * (R[n] - L[n]))
                   / (srvr * Ur[0] - slvl * Ul[0]);
    double bnint = (sr * Ur[bn] - sl * Ul[bn]) / (sr - sl);
    double rholl = Ul[0] * slvl * oneoslsm;
    double rhorr = Ur[0] * srvr * oneosrsm;

    /* degenerate-safe left ** state (hlldx.h:222-247) */
    double sgn = (fabs(fabs(Ul[0] * slvl * (sl - sm) - bnint * bnint) - 1.0e-8 * bnint * bnint)
                  / (fabs(Ul[0] * slvl * (sl - sm) - bnint * bnint) - 1.0e-8 * bnint * bnint));
    double denominator = ((1.0 / (Ul[0] * slvl * (sl - sm) - bnint * bnint) + 1.0)
                          + (1.0 / (Ul[0] * slvl * (sl - sm) - bnint * bnint) - 1.0) * sgn) * 0.5;
    double numerator = ((((Ul[0] * slvl * slvl - bnint * bnint) + 1.0)
                         + ((Ul[0] * slvl * slvl - bnint * bnint) - 1.0) * sgn) * 0.5);
    double vt1ll = L[t1] - (bnint * Ul[bt1] * (sm - L[n]) * ((denominator + denominator * sgn) * 0.5));
    double vt2ll = L[t2] - (bnint * Ul[bt2] * (sm - L[n]) * ((denominator + denominator * sgn) * 0.5));
    double bt1ll = Ul[bt1] * numerator * denominator;
    double bt2ll = Ul[bt2] * numerator * denominator;
    double vlldotbll = sm * bnint + vt1ll * bt1ll + vt2ll * bt2ll;

    /* right ** state (hlldx.h:295-320) */
    sgn = (fabs(fabs(Ur[0] * srvr * (sr - sm) - bnint * bnint) - 1.0e-8 * bnint * bnint)
           / (fabs(Ur[0] * srvr * (sr - sm) - bnint * bnint) - 1.0e-8 * bnint * bnint));
    denominator = ((1.0 / (Ur[0] * srvr * (sr - sm) - bnint * bnint) + 1.0)
                   + (1.0 / (Ur[0] * srvr * (sr - sm) - bnint * bnint) - 1.0) * sgn) * 0.5;
    numerator = ((((Ur[0] * srvr * srvr - bnint * bnint) + 1.0)
                  + ((Ur[0] * srvr * srvr - bnint * bnint) - 1.0) * sgn) * 0.5);
    double vt1rr = R[t1] - (bnint * Ur[bt1] * (sm - R[n]) * ((denominator + denominator * sgn) * 0.5));
    double vt2rr = R[t2] - (bnint * Ur[bt2] * (sm - R[n]) * ((denominator + denominator * sgn) * 0.5));
    double bt1rr = Ur[bt1] * numerator * denominator;
    double bt2rr = Ur[bt2] * numerator * denominator;
    double vrrdotbrr = sm * bnint + vt1rr * bt1rr + vt2rr * bt2rr;

    double enll = (slvl * Ul[7] - ptl * L[n] + ptint * sm + bnint * (vldotbl - vlldotbll)) * oneoslsm;
    double enrr = (srvr * Ur[7] - ptr * R[n] + ptint * sm + bnint * (vrdotbr - vrrdotbrr)) * oneosrsm;
    double sqrtrholl = sqrt(rholl);
    double sqrtrhorr = sqrt(rhorr);
    double sll = sm - fabs(bnint) / sqrtrholl;
    double srr = sm + fabs(bnint) / sqrtrhorr;

    double vv[4], bb[4];
    vv[n] = sm; bb[bn - 3] = bnint;
    if (sm >= 0.0 && sll >= 0.0) {
        vv[t1] = vt1ll; vv[t2] = vt2ll; bb[t1] = bt1ll; bb[t2] = bt2ll;
        star_flux(dir, vlldotbll, rholl, vv, bb, enll, ptint, r, Fo);
        return;
    }
    if (sm < 0.0 && srr <= 0.0) {
        vv[t1] = vt1rr; vv[t2] = vt2rr; bb[t1] = bt1rr; bb[t2] = bt2rr;
        star_flux(dir, vrrdotbrr, rhorr, vv, bb, enrr, ptint, r, Fo);
        return;
    }
    sgn = fabs(bnint) / bnint;
    double oneosqrtrho = 1.0 / (sqrtrholl + sqrtrhorr);
    double vt1int = (sqrtrholl * vt1ll + sqrtrhorr * vt1rr + (bt1rr - bt1ll) * sgn) * oneosqrtrho;
    double vt2int = (sqrtrholl * vt2ll + sqrtrhorr * vt2rr + (bt2rr - bt2ll) * sgn) * oneosqrtrho;
    double bt1int = (sqrtrholl * bt1rr + sqrtrhorr * bt1ll + sqrtrholl * sqrtrhorr * (vt1rr - vt1ll) * sgn) * oneosqrtrho;
    double bt2int = (sqrtrholl * bt2rr + sqrtrhorr * bt2ll + sqrtrholl * sqrtrhorr * (vt2rr - vt2ll) * sgn) * oneosqrtrho;
    double vintdotbint = sm * bnint + vt1int * bt1int + vt2int * bt2int;
    vv[t1] = vt1int; vv[t2] = vt2int; bb[t1] = bt1int; bb[t2] = bt2int;
    if (sm >= 0.0) {
        double enlll = enll - sqrtrholl * (vlldotbll - vintdotbint) * sgn;
        star_flux(dir, vintdotbint, rholl, vv, bb, enlll, ptint, r, Fo);
    } else {
        double enrrr = enrr + sqrtrhorr * (vrrdotbrr - vintdotbint) * sgn;
        star_flux(dir, vintdotbint, rhorr, vv, bb, enrrr, ptint, r, Fo);
    }
}

/* HLL: hllx.h:42-162, hlly.h, hllz.h */
static void hll_face(int dir, const double *L, const double *R, double r, double oneor, double *Fo)
{
    int n = 1 + dir, bn = 4 + dir;
    double Ul[9], Ur[9], Fl[8], Fr[8];
    double v2 = L[1] * L[1] + L[2] * L[2] + L[3] * L[3];
    double b2 = L[4] * L[4] + L[5] * L[5] + L[6] * L[6];
    double vdotb = L[1] * L[4] + L[2] * L[5] + L[3] * L[6];
    prim_to_cons(L, v2, b2, r, Ul);
    side_flux(dir, L, Ul, b2, vdotb, r, oneor, Fl);
    double gmpr = GM * L[7];
    double vfl = sqrt(((b2 + gmpr) + sqrt((b2 + gmpr) * (b2 + gmpr) - 4.0 * gmpr * L[bn] * L[bn])) / (2.0 * L[0]));
    v2 = R[1] * R[1] + R[2] * R[2] + R[3] * R[3];
    b2 = R[4] * R[4] + R[5] * R[5] + R[6] * R[6];
    vdotb = R[1] * R[4] + R[2] * R[5] + R[3] * R[6];
    prim_to_cons(R, v2, b2, r, Ur);
    side_flux(dir, R, Ur, b2, vdotb, r, oneor, Fr);
    gmpr = GM * R[7];
    double vfr = sqrt(((b2 + gmpr) + sqrt((b2 + gmpr) * (b2 + gmpr) - 4.0 * gmpr * R[bn] * R[bn])) / (2.0 * R[0]));
    double sl = rmin(L[n], R[n]) - rmax(vfl, vfr);
    double sr = rmax(L[n], R[n]) + rmax(vfl, vfr);
    int m;
    if (sl >= 0.0) {
        for (m = 0; m < 8; m++) Fo[m] = Fl[m];
    } else if (sr >= 0.0) {
        for (m = 0; m < 8; m++)
            Fo[m] = (sr * Fl[m] - sl * Fr[m] + sr * sl * (Ur[m] - Ul[m])) / (sr - sl);
    } else {
        for (m = 0; m < 8; m++) Fo[m] = Fr[m];
    }
}

/* Riemann sweep over all faces + GLM flux (hlldx.h:482-494, hlldy.h:490-503,
 * hlldz.h:486-498; hllx.h:167-179) */
static void riemann(orc_ctx *o, int dir, double *Fd)
{
    int ixmax1 = o->ixmax - 1, jymax1 = o->jymax - 1, kzmax1 = o->kzmax - 1;
    int bn = 4 + dir;
    double ch = o->ch;
    int i;
#pragma omp parallel for
    for (i = 0; i < ixmax1; i++) {
        double r = dir == 0 ? o->xm[i] : o->x[i];
        double oneor = o->oneox[i];
        for (int j = 0; j < jymax1; j++) {
            for (int k = 0; k < kzmax1; k++) {
                size_t q = IDX(o, i, j, k);
                double L[9], R[9], Fo[8];
                for (int m = 0; m < 9; m++) {
                    L[m] = o->Vl[(size_t)m * o->nc + q];
                    R[m] = o->Vr[(size_t)m * o->nc + q];
                }
                if (o->p.solver == 0) hlld_face(dir, L, R, r, oneor, Fo);
                else hll_face(dir, L, R, r, oneor, Fo);
                for (int m = 0; m < 8; m++) Fd[(size_t)m * o->nc + q] = Fo[m];
                Fd[(size_t)bn * o->nc + q] += 0.5 * (L[8] + R[8] + ch * (L[bn] - R[bn]));
                Fd[8 * o->nc + q] = 0.5 * ch * (ch * (L[bn] + R[bn]) + (L[8] - R[8]));
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* source.h:26-134 (SpiralGravityCooling); AxiGravityCooling (:143-204) and  */
/* AxiGravity (:207-266) are its i < irin branch everywhere, with cooling on */
/* or off; UniformGz (:269-305); NoSource (:308-349)                         */
/* ------------------------------------------------------------------------ */
static void source_other(orc_ctx *o)
{
    int i;
#pragma omp parallel for
    for (i = 0; i < o->ixmax; i++) {
        double oxi = o->oneox[i];
        for (int j = 0; j < o->jymax; j++)
            for (int k = 0; k < o->kzmax; k++) {
                size_t q = IDX(o, i, j, k), nc = o->nc;
                const double *V = o->V;
                double v0 = V[q], v1 = V[nc + q], v2 = V[2 * nc + q], v3 = V[3 * nc + q];
                double v4 = V[4 * nc + q], v5 = V[5 * nc + q], v6 = V[6 * nc + q], v7 = V[7 * nc + q];
                double *S = o->S;
                for (int m = 0; m < 9; m++) S[m * nc + q] = 0.0;
                if (o->p.source == 2) {
                    S[3 * nc + q] = -v0 * 1.0;
                    S[7 * nc + q] = -v3 * v0 * 1.0;
                } else {
                    S[nc + q] = (v0 * v2 * v2 - v5 * v5 + (v7 + 0.5 * (v4 * v4 + v5 * v5 + v6 * v6))) * oxi;
                    S[5 * nc + q] = (v5 * v1 - v2 * v4) * oxi;
                }
            }
    }
}

static void source(orc_ctx *o)
{
    const orc_params *p = &o->p;
    double omegasp = p->omegasp;
    int i;
    if (p->source >= 2) { source_other(o); return; }
#pragma omp parallel for
    for (i = 0; i < o->ixmax; i++) {
        double xi = o->x[i], oxi = o->oneox[i];
        for (int j = 0; j < o->jymax; j++) {
            for (int k = 0; k < o->kzmax; k++) {
                size_t q = IDX(o, i, j, k), nc = o->nc;
                const double *V = o->V;
                double v0 = V[q], v1 = V[nc + q], v2 = V[2 * nc + q], v3 = V[3 * nc + q];
                double v4 = V[4 * nc + q], v5 = V[5 * nc + q], v6 = V[6 * nc + q], v7 = V[7 * nc + q];
                double *S = o->S;
                int cl = cool(o, v0, v7);
                S[q] = 0.0;
                if (i < o->irin || p->source == 1) {
                    double gx = o->graxi[q], gz = o->graxi[2 * nc + q];
                    S[nc + q] = ((v0 * v2 * v2 - v5 * v5 + (v7 + 0.5 * (v4 * v4 + v5 * v5 + v6 * v6))) * oxi
                                 + v0 * gx + v0 * omegasp * omegasp * xi + (2.0 * v0 * v2 * omegasp));
                    S[2 * nc + q] = xi * (-2.0 * v0 * v1 * omegasp);
                    S[3 * nc + q] = v0 * gz;
                    S[7 * nc + q] = (v0 * (v1 * gx + v3 * gz) - (v0 * v0 * cl) + v0 * xi * v1 * omegasp * omegasp);
                } else {
                    double gx = o->gr[q], gy = o->gr[nc + q], gz = o->gr[2 * nc + q];
                    S[nc + q] = ((v0 * v2 * v2 - v5 * v5 + (v7 + 0.5 * (v4 * v4 + v5 * v5 + v6 * v6))) * oxi
                                 + v0 * gx + v0 * omegasp * omegasp * xi + (2.0 * v0 * v2 * omegasp));
                    S[2 * nc + q] = xi * (v0 * gy - (2.0 * v0 * v1 * omegasp));
                    S[3 * nc + q] = v0 * gz;
                    S[7 * nc + q] = (v0 * (v1 * gx + v2 * gy + v3 * gz) - (v0 * v0 * cl) + v0 * xi * v1 * omegasp * omegasp);
                }
                S[4 * nc + q] = 0.0;
                S[5 * nc + q] = (v5 * v1 - v2 * v4) * oxi;
                S[6 * nc + q] = 0.0;
                S[8 * nc + q] = 0.0;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* conservative update of one stage                                          */
/* kind 0: U1=U-dt L   (halfstep.h:97-104, firststep.h:104-111)              */
/* kind 1: U1=(3U+U1-dt L)/4       (secondstep.h:294-301)                    */
/* kind 2: U=(U+2(U1-dt L))/3      (thirdstep.h:484-493)                     */
/* kind 3: U=(U+U1-dt L)/2         (fullstep.h:279-286)                      */
/* ------------------------------------------------------------------------ */
static void update(orc_ctx *o, int kind)
{
    size_t pl = (size_t)o->ixmax * o->kzmax;
    double dt = o->dt;
    int m;
#pragma omp parallel for collapse(2)
    for (m = 0; m < 9; m++) {
        for (int i = 1; i < o->ixmax - 1; i++) {
            for (int j = 1; j < o->jymax - 1; j++) {
                for (int k = 1; k < o->kzmax - 1; k++) {
                    size_t q = IDX(o, i, j, k), mq = (size_t)m * o->nc + q;
                    size_t gk = (size_t)i * o->kzmax + k;
                    double g1 = o->g[gk], g2 = o->g[pl + gk], g3 = o->g[2 * pl + gk];
                    double g4 = o->g[3 * pl + gk], g5 = o->g[4 * pl + gk], g6 = o->g[5 * pl + gk];
                    size_t si = (size_t)o->jymax * o->kzmax, sj = (size_t)o->kzmax;
                    double div = ((g2 * o->F[mq] - g1 * o->F[mq - si])
                                  + (g4 * o->G[mq] - g3 * o->G[mq - sj])
                                  + (g6 * o->H[mq] - g5 * o->H[mq - 1]));
                    double s = o->S[mq];
                    if (kind == 0)
                        o->U1[mq] = o->U[mq] - dt * div + dt * s;
                    else if (kind == 1)
                        o->U1[mq] = 0.25 * (3.0 * o->U[mq] + o->U1[mq] - dt * div + dt * s);
                    else if (kind == 2)
                        o->U[mq] = ONEO3 * (o->U[mq] + 2.0 * (o->U1[mq] - dt * div + dt * s));
                    else
                        o->U[mq] = 0.5 * (o->U[mq] + o->U1[mq] - dt * div + dt * s);
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* boundary fills of U (xboundary.h, yboundary.h, zboundary.h,               */
/* centralboundary.h)                                                        */
/* ------------------------------------------------------------------------ */
static void bc_y_periodic(orc_ctx *o, double *Ud)   /* yboundary.h:97-154 */
{
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->ixmax; i++)
            for (int k = 0; k < o->kzmax; k++)
                A4(o, Ud, m, i, 0, k) = A4(o, Ud, m, i, o->jymax - 2, k);
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->ixmax; i++)
            for (int k = 0; k < o->kzmax; k++)
                A4(o, Ud, m, i, o->jymax - 1, k) = A4(o, Ud, m, i, 1, k);
}

static const double AXIS_SIGN[9] = {1.0, -1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 1.0, 1.0};

static void bc_x_axis(orc_ctx *o, double *Ud)      /* xboundary.h:33-72 */
{
    int half = o->jy / 2;
    int j;
#pragma omp parallel for
    for (j = 0; j < half + 1; j++)
        for (int k = 0; k < o->kzmax; k++)
            for (int m = 0; m < 9; m++) {
                double v = A4(o, Ud, m, 1, j + half, k);
                A4(o, Ud, m, 0, j, k) = AXIS_SIGN[m] < 0.0 ? -v : v;
            }
#pragma omp parallel for
    for (j = half + 1; j < o->jymax; j++)
        for (int k = 0; k < o->kzmax; k++)
            for (int m = 0; m < 9; m++) {
                double v = A4(o, Ud, m, 1, j - half, k);
                A4(o, Ud, m, 0, j, k) = AXIS_SIGN[m] < 0.0 ? -v : v;
            }
}

static void bc_x_right_free(orc_ctx *o, double *Ud)  /* xboundary.h:322-346 */
{
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int j = 0; j < o->jymax; j++)
            for (int k = 0; k < o->kzmax; k++)
                A4(o, Ud, m, o->ixmax - 1, j, k) = A4(o, Ud, m, o->ixmax - 2, j, k);
}

static void bc_z_left_antisym(orc_ctx *o, double *Ud)  /* zboundary.h:67-96 */
{
    int i;
#pragma omp parallel for
    for (i = 0; i < o->ixmax; i++)
        for (int j = 0; j < o->jymax; j++) {
            for (int m = 0; m < 9; m++) {
                double v = A4(o, Ud, m, i, j, 2);
                A4(o, Ud, m, i, j, 0) = m == 3 ? -v : v;
            }
            A4(o, Ud, 3, i, j, 1) = 0.0;
        }
}

static void bc_z_right_free(orc_ctx *o, double *Ud)   /* zboundary.h:203-226 */
{
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->ixmax; i++)
            for (int j = 0; j < o->jymax; j++)
                A4(o, Ud, m, i, j, o->kzmax - 1) = A4(o, Ud, m, i, j, o->kzmax - 2);
}

static void bc_z_periodic(orc_ctx *o, double *Ud)     /* zboundary.h:105-161 */
{
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->ixmax; i++)
            for (int j = 0; j < o->jymax; j++)
                A4(o, Ud, m, i, j, 0) = A4(o, Ud, m, i, j, o->kzmax - 2);
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->ixmax; i++)
            for (int j = 0; j < o->jymax; j++)
                A4(o, Ud, m, i, j, o->kzmax - 1) = A4(o, Ud, m, i, j, 1);
}

static void absorb_x_right(orc_ctx *o, double *Ud)    /* xboundary.h:124-149 */
{
    int m;
    int i0 = o->ixmax - 1 - 10;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = i0; i < o->ixmax; i++)
            for (int j = 0; j < o->jymax; j++)
                for (int k = 0; k < o->kzmax; k++) {
                    size_t mq = (size_t)m * o->nc + IDX(o, i, j, k);
                    Ud[mq] -= (o->xabs[i - i0] * (Ud[mq] - o->Uinit[mq]));
                }
}

static void absorb_central(orc_ctx *o, double *Ud)    /* centralboundary.h:27-52 */
{
    int m;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->irin + 1; i++)
            for (int j = 0; j < o->jymax; j++)
                for (int k = 0; k < o->kzmax; k++) {
                    size_t mq = (size_t)m * o->nc + IDX(o, i, j, k);
                    Ud[mq] -= (o->cabs[(size_t)i * o->kzmax + k] * (Ud[mq] - o->Uinit[mq]));
                }
}

static void absorb_z_right(orc_ctx *o, double *Ud)    /* zboundary.h:33-58 */
{
    int m;
    int k0 = o->kzmax - 1 - 10;
#pragma omp parallel for
    for (m = 0; m < 9; m++)
        for (int i = 0; i < o->ixmax; i++)
            for (int j = 0; j < o->jymax; j++)
                for (int k = k0; k < o->kzmax; k++) {
                    size_t mq = (size_t)m * o->nc + IDX(o, i, j, k);
                    Ud[mq] -= (o->zabs[k - k0] * (Ud[mq] - o->Uinit[mq]));
                }
}

/* ------------------------------------------------------------------------ */
/* utov.h:24-68 and check.h:23-188                                           */
/* ------------------------------------------------------------------------ */
static void utov(orc_ctx *o, const double *Ud)
{
    int i;
#pragma omp parallel for
    for (i = 0; i < o->ixmax; i++) {
        double ox = o->oneox[i];
        for (int j = 0; j < o->jymax; j++)
            for (int k = 0; k < o->kzmax; k++) {
                size_t q = IDX(o, i, j, k), nc = o->nc;
                double u0 = Ud[q], u1 = Ud[nc + q], u2 = Ud[2 * nc + q], u3 = Ud[3 * nc + q];
                double u4 = Ud[4 * nc + q], u5 = Ud[5 * nc + q], u6 = Ud[6 * nc + q];
                double oneorho = 1.0 / u0;
                double b2 = u4 * u4 + u5 * u5 + u6 * u6;
                double r2v2 = u1 * u1 + u2 * u2 * ox * ox + u3 * u3;
                double *V = o->V;
                V[q] = u0;
                V[nc + q] = u1 * oneorho;
                V[2 * nc + q] = u2 * oneorho * ox;
                V[3 * nc + q] = u3 * oneorho;
                V[4 * nc + q] = u4;
                V[5 * nc + q] = u5;
                V[6 * nc + q] = u6;
                V[7 * nc + q] = GM1 * (Ud[7 * nc + q] - 0.5 * (r2v2 * oneorho + b2));
                V[8 * nc + q] = Ud[8 * nc + q];
            }
    }
}

static void check(orc_ctx *o, double *Ud)
{
    int rhoflag = 0, prflag = 0, oneobetaflag = 0;
    const double prcr = o->p.prcr, betacr = o->p.betacr;
    const double oneobetacr = (1.0 / betacr);
    int i;
#pragma omp parallel for reduction(+ : rhoflag, prflag, oneobetaflag)
    for (i = 0; i < o->ixmax; i++) {
        double xi = o->x[i];
        for (int j = 0; j < o->jymax; j++)
            for (int k = 0; k < o->kzmax; k++) {
                size_t q = IDX(o, i, j, k), nc = o->nc;
                double *V = o->V;
                double v2 = V[2 * nc + q] * V[2 * nc + q];
                double b2 = (V[4 * nc + q] * V[4 * nc + q] + V[5 * nc + q] * V[5 * nc + q]
                             + V[6 * nc + q] * V[6 * nc + q]);
                if (V[q] < o->rhofloor[q]) {
                    rhoflag++;
                    V[q] = o->rhofloor[q];
                    V[nc + q] = 0.0;
                    V[3 * nc + q] = 0.0;
                    Ud[q] = V[q];
                    Ud[nc + q] = 0.0;
                    Ud[2 * nc + q] = xi * V[q] * V[2 * nc + q];
                    Ud[3 * nc + q] = 0.0;
                    Ud[7 * nc + q] = 0.5 * (V[q] * v2 + b2) + ONEOGM1 * V[7 * nc + q];
                }
                double prfloor = V[q] * prcr;
                if (V[7 * nc + q] < prfloor) {
                    prflag++;
                    V[nc + q] = 0.0;
                    V[3 * nc + q] = 0.0;
                    V[7 * nc + q] = prfloor;
                    Ud[nc + q] = 0.0;
                    Ud[3 * nc + q] = 0.0;
                    Ud[7 * nc + q] = (0.5 * (V[q] * v2 + b2) + ONEOGM1 * V[7 * nc + q]);
                }
                double oneobeta = 0.5 * b2 / V[7 * nc + q];
                if (oneobeta > oneobetacr) {
                    oneobetaflag++;
                    V[q] = betacr * oneobeta * V[q];
                    V[nc + q] = 0.0;
                    V[3 * nc + q] = 0.0;
                    V[7 * nc + q] = betacr * oneobeta * V[7 * nc + q];
                    Ud[q] = V[q];
                    Ud[nc + q] = 0.0;
                    Ud[2 * nc + q] = xi * V[q] * V[2 * nc + q];
                    Ud[3 * nc + q] = 0.0;
                    Ud[7 * nc + q] = (0.5 * (V[q] * v2 + b2) + ONEOGM1 * V[7 * nc + q]);
                }
            }
    }
    o->counters[0] = rhoflag; o->counters[1] = prflag; o->counters[2] = oneobetaflag;
}

/* ------------------------------------------------------------------------ */
/* stages and step                                                           */
/* ------------------------------------------------------------------------ */
static void fluxes(orc_ctx *o)
{
    limiter(o, 0); riemann(o, 0, o->F);
    limiter(o, 1); riemann(o, 1, o->G);
    limiter(o, 2); riemann(o, 2, o->H);
    source(o);
}

/* stage: 1..3 = FirstStep/SecondStep/ThirdStep; 4,5 = Halfstep/Fullstep */
static void stage(orc_ctx *o, int which)
{
    int rk2 = which >= 4;
    double *dst = (which == 3 || which == 5) ? o->U : o->U1;
    glm_damp(o, which == 1 || which == 4 ? o->U : o->U1);
    fluxes(o);
    update(o, which == 1 || which == 4 ? 0 : which == 2 ? 1 : which == 3 ? 2 : 3);
    bc_y_periodic(o, dst);
    bc_x_axis(o, dst);
    bc_x_right_free(o, dst);
    if (rk2) { bc_z_left_antisym(o, dst); bc_z_right_free(o, dst); }
    else bc_z_periodic(o, dst);
    if (which == 3 || which == 5) {
        absorb_x_right(o, dst);
        absorb_central(o, dst);
        if (which == 5) absorb_z_right(o, dst);
    }
    utov(o, dst);
    check(o, dst);
}

int orc_step(orc_ctx *o, double *t, double *dt, double *ch, int *counters)
{
    orc_setdt(o, dt, ch, NULL);
    if (isinf(o->dt) || o->dt < o->p.dtmin) return 1;
    o->t = *t;
    if (o->p.gravity) orc_spiral_gravity(o, *t);
    if (o->p.scheme == 2) {
        o->psicoef = exp(-o->dt * o->ch * ONEOCR * 0.5);     /* tvdrungekutta.h:34 */
        stage(o, 4);
        stage(o, 5);
    } else {
        o->psicoef = exp(-o->dt * o->ch * ONEOCR * ONEO3);   /* tvdrungekutta.h:33 */
        stage(o, 1);
        stage(o, 2);
        stage(o, 3);
    }
    counters[0] = o->counters[0]; counters[1] = o->counters[1]; counters[2] = o->counters[2];
    *t = *t + o->dt;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* probes                                                                    */
/* ------------------------------------------------------------------------ */
void orc_set_dtch(orc_ctx *o, double dt, double ch, double psicoef)
{
    o->dt = dt; o->ch = ch; o->psicoef = psicoef;
}

static void to_face_layout(const orc_ctx *o, const double *src, double *dst)
{
    int a = o->ixmax - 1, b = o->jymax - 1, c = o->kzmax - 1;
    for (int m = 0; m < 9; m++)
        for (int i = 0; i < a; i++)
            for (int j = 0; j < b; j++)
                for (int k = 0; k < c; k++)
                    dst[(((size_t)m * a + i) * b + j) * c + k] = A4(o, src, m, i, j, k);
}

void orc_limiter(orc_ctx *o, int dir, double *Vl, double *Vr)
{
    memset(o->Vl, 0, 9 * o->nc * sizeof(double));
    memset(o->Vr, 0, 9 * o->nc * sizeof(double));
    limiter(o, dir);
    to_face_layout(o, o->Vl, Vl);
    to_face_layout(o, o->Vr, Vr);
}

void orc_flux(orc_ctx *o, int dir, double *Fout)
{
    double *Fd = dir == 0 ? o->F : dir == 1 ? o->G : o->H;
    memset(Fd, 0, 9 * o->nc * sizeof(double));
    limiter(o, dir);
    riemann(o, dir, Fd);
    to_face_layout(o, Fd, Fout);
}

void orc_source(orc_ctx *o, double *S)
{
    source(o);
    memcpy(S, o->S, 9 * o->nc * sizeof(double));
}

void orc_utov_check(orc_ctx *o, double *U, double *V, int *counters)
{
    memcpy(o->U, U, 9 * o->nc * sizeof(double));
    utov(o, o->U);
    check(o, o->U);
    memcpy(U, o->U, 9 * o->nc * sizeof(double));
    memcpy(V, o->V, 9 * o->nc * sizeof(double));
    counters[0] = o->counters[0]; counters[1] = o->counters[1]; counters[2] = o->counters[2];
}
