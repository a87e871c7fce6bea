/*
 * mhd_io.c -- the reference's checkpoint files and restart sequence on the
 * host, so a host that keeps its own I/O can hand it to the library and one
 * that uses the library's asynchronous checkpoint gets the same bytes.
 *
 *   BinaryOutput()  output.h:1202-1414    -> mhd_binary_output()
 *   RestartRead()   restartread.h:9-143   -> mhd_restart_read() + mhd_vtou()
 *                                            + mhd_check()
 *   SaveInitial()   saveinitial.h:18-50   -> mhd_save_initial()
 *   restart branch  main.c:244-272        -> mhd_restart()
 *   GNUOutputCylinder() output.h:25-150   -> mhd_gnu_output_cylinder()
 *   GDLOutputCylinder() output.h:280-390  -> mhd_gdl_output_cylinder()
 *
 * File format (one directory per output number, relative to a root
 * directory; the reference uses the working directory):
 *   <root>/<n>/GridTime.dat   text "%d\t%d\t%d\t%.3e": ixmax, jymax, kzmax, t
 *   <root>/<n>/r, phi, z      raw FP64 cell centres x[ixmax], y[jymax], z[kzmax]
 *   <root>/<n>/rho, vr, vphi, vz, br, bphi, bz, pr, psi
 *                             raw FP64 V[m][ixmax][jymax][kzmax], ghosts included
 * in the host's byte order, as fwrite() of the reference's arrays leaves them.
 * Compiled with -ffp-contract=off.
 */
#include "mhd_gpu.h"
#include "mhd_internal.h"

#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

/* output.h:1289-1409 and restartread.h:17-121: file name of V[m] */
static const char *const vname[9] = {"rho", "vr", "vphi", "vz", "br", "bphi", "bz", "pr", "psi"};

static int write_raw(const char *dir, const char *name, const double *a, size_t n)
{
    char path[4096];
    if (snprintf(path, sizeof path, "%s/%s", dir, name) >= (int)sizeof path) return MHD_ERR_ARG;
    FILE *f = fopen(path, "wb");
    if (!f) return MHD_ERR_IO;
    size_t w = fwrite(a, sizeof(double), n, f);
    int rc = fclose(f);
    return (w == n && rc == 0) ? MHD_OK : MHD_ERR_IO;
}

static int read_raw(const char *dir, const char *name, double *a, size_t n)
{
    char path[4096];
    if (snprintf(path, sizeof path, "%s/%s", dir, name) >= (int)sizeof path) return MHD_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return MHD_ERR_IO;
    size_t r = fread(a, sizeof(double), n, f);
    fclose(f);
    return r == n ? MHD_OK : MHD_ERR_IO;
}

int mhd_binary_output_arrays(const char *root, int nout, double t, int ix, int jy, int kz, const double *x,
                             const double *y, const double *z, const double *V)
{
    if (!root || !x || !y || !z || !V || ix < 1 || jy < 1 || kz < 1 || nout < 0) return MHD_ERR_ARG;
    const size_t ixmax = (size_t)ix + 2, jymax = (size_t)jy + 2, kzmax = (size_t)kz + 2;
    const size_t nc = ixmax * jymax * kzmax;
    char dir[4096];
    if (snprintf(dir, sizeof dir, "%s/%d", root, nout) >= (int)sizeof dir) return MHD_ERR_ARG;
    /* output.h:1208-1210: the same permission bits; an existing directory is reused */
    if (mkdir(dir, S_IRUSR | S_IWUSR | S_IXUSR | S_IRGRP | S_IWGRP | S_IXGRP | S_IROTH | S_IXOTH) != 0 &&
        errno != EEXIST)
        return MHD_ERR_IO;
    char path[4096];
    if (snprintf(path, sizeof path, "%s/GridTime.dat", dir) >= (int)sizeof path) return MHD_ERR_ARG;
    FILE *f = fopen(path, "w");
    if (!f) return MHD_ERR_IO;
    int pr = fprintf(f, "%d\t%d\t%d\t%.3e", (int)ixmax, (int)jymax, (int)kzmax, t);
    if (fclose(f) != 0 || pr < 0) return MHD_ERR_IO;
    int rc;
    if ((rc = write_raw(dir, "r", x, ixmax))) return rc;
    if ((rc = write_raw(dir, "phi", y, jymax))) return rc;
    if ((rc = write_raw(dir, "z", z, kzmax))) return rc;
    for (int m = 0; m < 9; m++)
        if ((rc = write_raw(dir, vname[m], V + (size_t)m * nc, nc))) return rc;
    return MHD_OK;
}

int mhd_binary_output(const char *root, int nout, double t, const mhd_grid *g, const double *V)
{
    if (!g) return MHD_ERR_ARG;
    return mhd_binary_output_arrays(root, nout, t, g->ix, g->jy, g->kz, g->x, g->y, g->z, V);
}

int mhd_restart_read(const char *root, int num, int ix, int jy, int kz, double *V)
{
    if (!root || !V || ix < 1 || jy < 1 || kz < 1 || num < 0) return MHD_ERR_ARG;
    const size_t nc = ((size_t)ix + 2) * ((size_t)jy + 2) * ((size_t)kz + 2);
    char dir[4096];
    if (snprintf(dir, sizeof dir, "%s/%d", root, num) >= (int)sizeof dir) return MHD_ERR_ARG;
    for (int m = 0; m < 9; m++) {
        int rc = read_raw(dir, vname[m], V + (size_t)m * nc, nc);
        if (rc) return rc;
    }
    return MHD_OK;
}

/* Check() (check.h:23-188) over every cell, ghosts included: density floor
 * rhofloor, pressure floor prcr*rho, and the plasma-beta floor betacr, each
 * zeroing v_r and v_z and rebuilding U from V; counters = cells caught by
 * each floor (rhoflag, prflag, oneobetaflag). */
int mhd_check(const mhd_grid *g, const mhd_params *p, double *U, double *V, const double *rhofloor,
              int counters[3])
{
    if (!g || !p || !U || !V || !rhofloor) return MHD_ERR_ARG;
    const size_t ixmax = (size_t)g->ix + 2, jymax = (size_t)g->jy + 2, kzmax = (size_t)g->kz + 2;
    const size_t nc = ixmax * jymax * kzmax, plane = jymax * kzmax;
    const double prcr = p->prcr, betacr = p->betacr, oneobetacr = 1.0 / p->betacr;
    int nrho = 0, npr = 0, nbeta = 0;
    for (size_t q = 0; q < nc; q++) {
        const double xi = g->x[q / plane];
        double *v0 = V + q, *v1 = V + nc + q, *v2 = V + 2 * nc + q, *v3 = V + 3 * nc + q;
        double *v7 = V + 7 * nc + q;
        const double vphi2 = (*v2) * (*v2);
        const double b2 = (V[4 * nc + q] * V[4 * nc + q] + V[5 * nc + q] * V[5 * nc + q] +
                           V[6 * nc + q] * V[6 * nc + q]);
        if (*v0 < rhofloor[q]) {
            nrho++;
            *v0 = rhofloor[q];
            *v1 = 0.0;
            *v3 = 0.0;
            U[q] = *v0;
            U[nc + q] = 0.0;
            U[2 * nc + q] = xi * (*v0) * (*v2);
            U[3 * nc + q] = 0.0;
            U[7 * nc + q] = 0.5 * ((*v0) * vphi2 + b2) + MHD_ONEOGM1 * (*v7);
        }
        const double prfloor = (*v0) * prcr;
        if (*v7 < prfloor) {
            npr++;
            *v1 = 0.0;
            *v3 = 0.0;
            *v7 = prfloor;
            U[nc + q] = 0.0;
            U[3 * nc + q] = 0.0;
            U[7 * nc + q] = (0.5 * ((*v0) * vphi2 + b2) + MHD_ONEOGM1 * (*v7));
        }
        const double oneobeta = 0.5 * b2 / (*v7);
        if (oneobeta > oneobetacr) {
            nbeta++;
            *v0 = betacr * oneobeta * (*v0);
            *v1 = 0.0;
            *v3 = 0.0;
            *v7 = betacr * oneobeta * (*v7);
            U[q] = *v0;
            U[nc + q] = 0.0;
            U[2 * nc + q] = xi * (*v0) * (*v2);
            U[3 * nc + q] = 0.0;
            U[7 * nc + q] = (0.5 * ((*v0) * vphi2 + b2) + MHD_ONEOGM1 * (*v7));
        }
    }
    if (counters) { counters[0] = nrho; counters[1] = npr; counters[2] = nbeta; }
    return MHD_OK;
}

int mhd_save_initial(const mhd_grid *g, double rhocr, const double *U, const double *V, double *Uinit,
                     double *Vinit, double *rhofloor)
{
    if (!g || !U || !V) return MHD_ERR_ARG;
    const size_t nc = ((size_t)g->ix + 2) * ((size_t)g->jy + 2) * ((size_t)g->kz + 2);
    if (Uinit) memcpy(Uinit, U, 9 * nc * sizeof(double));
    if (Vinit) memcpy(Vinit, V, 9 * nc * sizeof(double));
    if (rhofloor)
        for (size_t q = 0; q < nc; q++) rhofloor[q] = U[q] * rhocr;
    return MHD_OK;
}

int mhd_restart(const char *root, int nout, double tint, const mhd_grid *g, const mhd_params *p, double *U,
                double *V, double *Uinit, double *Vinit, double *rhofloor, double *t, double *tout)
{
    if (!g || !p || !U || !V || !Uinit || !Vinit || !rhofloor) return MHD_ERR_ARG;
    const size_t nc = ((size_t)g->ix + 2) * ((size_t)g->jy + 2) * ((size_t)g->kz + 2);
    int rc;
    /* main.c:250-251: RestartRead(0) with the floors not yet set, SaveInitial() */
    memset(rhofloor, 0, nc * sizeof(double));
    if ((rc = mhd_restart_read(root, 0, g->ix, g->jy, g->kz, V))) return rc;
    if ((rc = mhd_vtou(g, V, U))) return rc;
    if ((rc = mhd_check(g, p, U, V, rhofloor, NULL))) return rc;
    if ((rc = mhd_save_initial(g, p->rhocr, U, V, Uinit, Vinit, rhofloor))) return rc;
    /* main.c:258-270: RestartRead(nout), t and the next output time */
    if ((rc = mhd_restart_read(root, nout, g->ix, g->jy, g->kz, V))) return rc;
    if ((rc = mhd_vtou(g, V, U))) return rc;
    if ((rc = mhd_check(g, p, U, V, rhofloor, NULL))) return rc;
    if (t) *t = nout * tint;
    if (tout) *tout = (nout + 1) * tint;
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* text outputs for plotting                                                 */
/* ------------------------------------------------------------------------ */
static FILE *open_in(const char *root, const char *name)
{
    char path[4096];
    if (snprintf(path, sizeof path, "%s/%s", root, name) >= (int)sizeof path) return NULL;
    return fopen(path, "w");
}

/* one 1D cut: header, then x/y/z and rho vr vphi vz br bphi bz E p per cell */
static int write_cut(const char *root, const char *name, int nstep, double t, int h1, int h2, const double *coord,
                     size_t n, size_t q0, size_t stride, size_t nc, const double *U, const double *V)
{
    FILE *f = open_in(root, name);
    if (!f) return MHD_ERR_IO;
    int bad = fprintf(f, "#\t nstep=%d,\ttime=%.3e,\tj=%d,\tk=%d \n", nstep, t, h1, h2) < 0;
    bad |= fprintf(f, "#%s rho vx vy vz bx by bz en pr\n", name[3] == 'r' ? "x" : name[3] == 'p' ? "y" : "z") < 0;
    for (size_t c = 1; c + 1 < n && !bad; c++) {
        size_t q = q0 + c * stride;
        bad |= fprintf(f,
                       "%.3e\t"
                       "%.3e\t%.3e\t%.3e\t%.3e\t"
                       "%.3e\t%.3e\t%.3e\t%.3e\t"
                       "%.3e\n",
                       coord[c], V[q], V[nc + q], V[2 * nc + q], V[3 * nc + q], V[4 * nc + q], V[5 * nc + q],
                       V[6 * nc + q], U[7 * nc + q], V[7 * nc + q]) < 0;
    }
    bad |= fclose(f) != 0;
    return bad ? MHD_ERR_IO : MHD_OK;
}

/* GNUOutputCylinder (output.h:25-150): 1d-r-<nout>.dat along r at j=1, k=1;
 * 1d-phi-<nout>.dat along phi and 1d-z-<nout>.dat along z at the fixed
 * radial index 160 (so the grid needs ix >= 159), with the header and column
 * formats of the reference (E is the conserved total energy U[7]). */
int mhd_gnu_output_cylinder(const char *root, int nout, int nstep, double t, const mhd_grid *g, const double *U,
                            const double *V)
{
    if (!root || !g || !U || !V || nout < 0) return MHD_ERR_ARG;
    const size_t ixmax = (size_t)g->ix + 2, jymax = (size_t)g->jy + 2, kzmax = (size_t)g->kz + 2;
    const size_t nc = ixmax * jymax * kzmax;
    const int icut = 160;
    if (ixmax <= (size_t)icut + 1) return MHD_ERR_ARG;
    char name[64];
    int rc;
    snprintf(name, sizeof name, "1d-r-%d.dat", nout);
    if ((rc = write_cut(root, name, nstep, t, 1, 1, g->x, ixmax, 1 * kzmax + 1, jymax * kzmax, nc, U, V))) return rc;
    snprintf(name, sizeof name, "1d-phi-%d.dat", nout);
    if ((rc = write_cut(root, name, nstep, t, icut, 1, g->y, jymax, (size_t)icut * jymax * kzmax + 1, kzmax, nc, U,
                        V)))
        return rc;
    snprintf(name, sizeof name, "1d-z-%d.dat", nout);
    return write_cut(root, name, nstep, t, icut, 1, g->z, kzmax, ((size_t)icut * jymax + 1) * kzmax, 1, nc, U, V);
}

static int write_column(const char *root, const char *name, const double *a, size_t n)
{
    FILE *f = open_in(root, name);
    if (!f) return MHD_ERR_IO;
    int bad = 0;
    for (size_t c = 1; c + 1 < n && !bad; c++) bad |= fprintf(f, "%e\n", a[c]) < 0;
    bad |= fclose(f) != 0;
    return bad ? MHD_ERR_IO : MHD_OK;
}

/* GDLOutputCylinder (output.h:280-390): r.dat, phi.dat, z.dat (interior
 * centres), the k=1 slices 2d-density-rphi, 2d-pressure-rphi,
 * 2d-benergy-rphi (B^2/2) with j fastest, and the j=0 slice 2d-density-rz
 * with r fastest; one "%e" value per line. */
int mhd_gdl_output_cylinder(const char *root, int nout, const mhd_grid *g, const double *V)
{
    if (!root || !g || !V || nout < 0) return MHD_ERR_ARG;
    const size_t ixmax = (size_t)g->ix + 2, jymax = (size_t)g->jy + 2, kzmax = (size_t)g->kz + 2;
    const size_t nc = ixmax * jymax * kzmax;
    int rc;
    if ((rc = write_column(root, "r.dat", g->x, ixmax))) return rc;
    if ((rc = write_column(root, "phi.dat", g->y, jymax))) return rc;
    if ((rc = write_column(root, "z.dat", g->z, kzmax))) return rc;
    static const char *const slice[3] = {"2d-density-rphi", "2d-pressure-rphi", "2d-benergy-rphi"};
    for (int s = 0; s < 3; s++) {
        char name[64];
        snprintf(name, sizeof name, "%s-%d.dat", slice[s], nout);
        FILE *f = open_in(root, name);
        if (!f) return MHD_ERR_IO;
        int bad = 0;
        for (size_t i = 1; i + 1 < ixmax && !bad; i++)
            for (size_t j = 1; j + 1 < jymax && !bad; j++) {
                size_t q = (i * jymax + j) * kzmax + 1;
                double v = s == 0 ? V[q]
                         : s == 1 ? V[7 * nc + q]
                                  : 0.5 * (V[4 * nc + q] * V[4 * nc + q] + V[5 * nc + q] * V[5 * nc + q]
                                           + V[6 * nc + q] * V[6 * nc + q]);
                bad |= fprintf(f, "%e\n", v) < 0;
            }
        bad |= fclose(f) != 0;
        if (bad) return MHD_ERR_IO;
    }
    char name[64];
    snprintf(name, sizeof name, "2d-density-rz-%d.dat", nout);
    FILE *f = open_in(root, name);
    if (!f) return MHD_ERR_IO;
    int bad = 0;
    for (size_t k = 1; k + 1 < kzmax && !bad; k++)
        for (size_t i = 1; i + 1 < ixmax && !bad; i++) bad |= fprintf(f, "%e\n", V[(i * jymax + 0) * kzmax + k]) < 0;
    bad |= fclose(f) != 0;
    return bad ? MHD_ERR_IO : MHD_OK;
}
