/*
 * mhd_disc -- the reference's main program (main.c:224-398) on the GPU
 * through the C-ABI of libmhdgpu.so: the same grid, initial model, restart
 * branch, step loop, output schedule, messages and file formats, with
 * Setdt/SpiralGravity/TVDRK replaced by mhd_step() and BinaryOutput() by the
 * library's (optionally asynchronous) checkpoint.
 *
 *   mhd_disc [--root DIR] [--grid NRxNPHIxNZ] [--nstop N] [--tint T] [--tstop T]
 *            [--restart NOUT] [--fp32] [--sync-output] [--quiet]
 *
 * Defaults are the reference's input.h: the 240x64x200 stretched grid,
 * nstop 10000000, tint 0.05, tstop 40.0, a fresh start (restartsw 0), FP64.
 * --grid keeps the shipped spacing and stretching with other cell counts.
 * Exit status 0, or 1 after the reference's dt-guard message (main.c:331-334)
 * or any library error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mhd_gpu.h"

static int fail(const char *what, int rc)
{
    fprintf(stderr, "%s: %s (%d)\n", what, mhd_errstr(rc), rc);
    return 1;
}

int main(int argc, char **argv)
{
    const char *root = ".";
    int nr = 0, nphi = 0, nz = 0, nstop = 10000000, restart = -1, fp32 = 0, async = 1, quiet = 0;
    double tint = 0.05, tstop = 40.0;
    for (int a = 1; a < argc; a++) {
        if (!strcmp(argv[a], "--root") && a + 1 < argc) root = argv[++a];
        else if (!strcmp(argv[a], "--grid") && a + 1 < argc) {
            if (sscanf(argv[++a], "%dx%dx%d", &nr, &nphi, &nz) != 3) return fail("--grid", MHD_ERR_ARG);
        } else if (!strcmp(argv[a], "--nstop") && a + 1 < argc) nstop = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--tint") && a + 1 < argc) tint = atof(argv[++a]);
        else if (!strcmp(argv[a], "--tstop") && a + 1 < argc) tstop = atof(argv[++a]);
        else if (!strcmp(argv[a], "--restart") && a + 1 < argc) restart = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--fp32")) fp32 = 1;
        else if (!strcmp(argv[a], "--sync-output")) async = 0;
        else if (!strcmp(argv[a], "--quiet")) quiet = 1;
        else {
            fprintf(stderr, "unknown argument %s\n", argv[a]);
            return 1;
        }
    }

    /* CylindricalGrid() (main.c:232) */
    mhd_gridspec gs;
    mhd_gridspec_shipped(&gs);
    if (nr) { gs.ix = nr; gs.jy = nphi; gs.kz = nz; }
    size_t nstore = mhd_grid_storage(&gs);
    double *store = malloc(nstore * sizeof(double));
    mhd_grid g;
    int rc;
    if (!store) return fail("grid", MHD_ERR_NOMEM);
    if ((rc = mhd_grid_build(&gs, store, &g))) return fail("mhd_grid_build", rc);
    if (!quiet) printf("complete grid setting.\n");
    const size_t ixmax = (size_t)gs.ix + 2, jymax = (size_t)gs.jy + 2, kzmax = (size_t)gs.kz + 2;
    const size_t nc = ixmax * jymax * kzmax;
    /* the fixed potential (initialgravity.h; GalacticDisc3 sets the same) */
    double *gr = malloc(3 * ixmax * kzmax * sizeof(double));
    if (!gr) return fail("gravity", MHD_ERR_NOMEM);
    if ((rc = mhd_initial_gravity(&g, gr, gr + ixmax * kzmax, gr + 2 * ixmax * kzmax))) return fail("gravity", rc);
    g.Grxaxi = gr; g.Gryaxi = gr + ixmax * kzmax; g.Grzaxi = gr + 2 * ixmax * kzmax;

    mhd_params p;
    mhd_params_default(&p);
    p.precision = fp32 ? MHD_PREC_FP32 : MHD_PREC_FP64;

    double *U = malloc(9 * nc * sizeof(double)), *V = malloc(9 * nc * sizeof(double));
    double *Ui = malloc(9 * nc * sizeof(double)), *Vi = malloc(9 * nc * sizeof(double));
    double *rf = malloc(nc * sizeof(double));
    if (!U || !V || !Ui || !Vi || !rf) return fail("state", MHD_ERR_NOMEM);

    int nstep = 0, nout = 0;
    double t = 0.0, tout = tint;
    if (restart >= 0) {
        /* main.c:244-272: RestartRead(0), SaveInitial(), RestartRead(nout) */
        nout = restart;
        if ((rc = mhd_restart(root, nout, tint, &g, &p, U, V, Ui, Vi, rf, &t, &tout))) return fail("restart", rc);
    } else {
        /* GalacticDisc3() then BinaryOutput() (main.c:299-304) */
        if ((rc = mhd_ic_galactic_disc3(&g, &p, U, V, Ui, Vi, rf))) return fail("GalacticDisc3", rc);
        if ((rc = mhd_binary_output(root, nout, t, &g, V))) return fail("BinaryOutput", rc);
        if (!quiet) printf("%d step binary output complete.\n", nout);
    }
    if (!quiet) printf("complete model setting.\n");

    mhd_ctx *ctx;
    if ((rc = mhd_create(&g, &p, &ctx))) return fail("mhd_create", rc);
    if ((rc = mhd_upload(ctx, U, V, Ui, Vi, rf))) return fail("mhd_upload", rc);

    int status = 0;
    /* the step loop, main.c:316-393 */
    while (nstep < nstop + 1) {
        nstep++;
        if (!quiet) printf("nstep = %d\n", nstep);
        double dt, ch;
        int cnt[3];
        rc = mhd_step(ctx, &t, &dt, &ch, cnt);
        if (!quiet) printf("dt = %.3e\n", dt);
        if (rc == MHD_ERR_DT) {
            printf("stop due to small dt or inf. program is done.\n");
            status = 1;
            break;
        }
        if (rc) { status = fail("mhd_step", rc); break; }
        if (t > tout) {
            if (!quiet) printf("time=%e.\n output complete.\n", t);
            tout += tint;
            nout++;
            if (async) rc = mhd_checkpoint_begin(ctx, root, nout, t);
            else if (!(rc = mhd_download(ctx, NULL, V))) rc = mhd_binary_output(root, nout, t, &g, V);
            if (rc) { status = fail("BinaryOutput", rc); break; }
            if (!quiet) printf("%d step binary output complete.\n", nout);
        }
        if (t > tstop) {
            if (!quiet) printf("time is over %.3e.\n", tstop);
            break;
        }
    }
    rc = mhd_checkpoint_wait(ctx);
    if (rc && !status) status = fail("BinaryOutput", rc);
    mhd_destroy(ctx);
    free(U); free(V); free(Ui); free(Vi); free(rf); free(gr); free(store);
    return status;
}
