/*
 * mhd_batch.cu -- many independent discs of uneven sizes and parameters.
 *
 * This first form keeps one context per disc and steps the discs in turn,
 * each with its own dt (the reference has no batched driver; each disc is a
 * run of main.c:316-393).  A disc whose dt guard fires (main.c:331) stops and
 * reports MHD_ERR_DT in its status slot; the others continue.
 */
#include <new>
#include <vector>

#include "mhd_gpu.h"

struct mhd_batch {
    int n;
    std::vector<mhd_ctx *> ctx;
    std::vector<int> stopped;
};

extern "C" int mhd_batch_create(int n, const mhd_grid *grids, const mhd_params *params, mhd_batch **out)
{
    if (!out || n < 1 || !grids || !params) return MHD_ERR_ARG;
    *out = NULL;
    mhd_batch *b = new (std::nothrow) mhd_batch();
    if (!b) return MHD_ERR_NOMEM;
    b->n = n;
    b->ctx.assign(n, NULL);
    b->stopped.assign(n, 0);
    for (int i = 0; i < n; i++) {
        int rc = mhd_create(&grids[i], &params[i], &b->ctx[i]);
        if (rc) {
            mhd_batch_destroy(b);
            return rc;
        }
    }
    *out = b;
    return MHD_OK;
}

extern "C" void mhd_batch_destroy(mhd_batch *b)
{
    if (!b) return;
    for (mhd_ctx *c : b->ctx)
        if (c) mhd_destroy(c);
    delete b;
}

extern "C" int mhd_batch_upload(mhd_batch *b, int disc, const double *U, const double *V, const double *Uinit,
                                const double *Vinit, const double *rhofloor)
{
    if (!b || disc < 0 || disc >= b->n) return MHD_ERR_ARG;
    b->stopped[disc] = 0;
    return mhd_upload(b->ctx[disc], U, V, Uinit, Vinit, rhofloor);
}

extern "C" int mhd_batch_download(mhd_batch *b, int disc, double *U, double *V)
{
    if (!b || disc < 0 || disc >= b->n) return MHD_ERR_ARG;
    return mhd_download(b->ctx[disc], U, V);
}

extern "C" int mhd_batch_step(mhd_batch *b, int nsteps, double *t, int *status)
{
    if (!b || !t || nsteps < 0) return MHD_ERR_ARG;
    for (int s = 0; s < nsteps; s++)
        for (int i = 0; i < b->n; i++) {
            if (b->stopped[i]) continue;
            double dt, ch;
            int cnt[3];
            int rc = mhd_step(b->ctx[i], &t[i], &dt, &ch, cnt);
            if (rc == MHD_ERR_DT) b->stopped[i] = 1;
            else if (rc) return rc;
        }
    if (status)
        for (int i = 0; i < b->n; i++) status[i] = b->stopped[i] ? MHD_ERR_DT : MHD_OK;
    return MHD_OK;
}

extern "C" int mhd_batch_tune(mhd_batch *b, int *best)
{
    if (!b || !best) return MHD_ERR_ARG;
    best[0] = 1; best[1] = 1; best[2] = 128; best[3] = 128;
    return MHD_OK;
}
