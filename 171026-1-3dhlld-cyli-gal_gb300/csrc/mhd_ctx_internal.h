/*
 * mhd_ctx_internal.h -- the context object behind the C-ABI, shared by the
 * context code (mhd_ctx.cu) and the batched form (mhd_batch.cu).
 */
#ifndef MHD_CTX_INTERNAL_H
#define MHD_CTX_INTERNAL_H

#include <cuda_runtime.h>

#include <string>
#include <thread>
#include <vector>

#include "mhd_launch.h"

#define NSTAGE 4   /* staging buffers (and copy streams) of the precision form's host transfers */
#define MHD_MAX_SLABS 64   /* slabs of the pipelined split stage (stage shape 3) */

struct mhd_ctx {
    int device;
    int nsm;                     /* multiprocessors of the device */
    cudaStream_t st;
    cudaStream_t st_aux;         /* the z boundary faces beside the interior z faces */
    cudaEvent_t ev_fork, ev_join;
    /* stage shape 3: the update of each slab of i planes on its own stream
     * (highest priority) beside the fluxes of the following slabs */
    cudaStream_t st_upd;
    cudaEvent_t ev_slab[MHD_MAX_SLABS], ev_upd;
    mhd_params p;
    int ix, jy, kz, ixmax, jymax, kzmax, irin;
    long long nc;
    int fp32;
    size_t esz;
    mhd::Geom G;
    double *dtab;
    float *ftab;
    void *U, *U1, *Va, *Vb, *Uinit, *Vinit, *rhofloor, *F, *Gf, *H, *Uraw;
    void *Zs;                    /* the split stage's z walk: 18 values per (i,j) row (last-face slots) */
    void *Hb;                    /* the split stage's last z face of each (i,j) row, [9][rows] */
    /* pair-state form (MHD_PREC_FP32X2): the low words of U, U1 and Uraw */
    int pair;
    float *Ulo, *U1lo, *Urawlo;
    int vcur;
    /* stage shape: fused = one kernel for fluxes + update (else the four
     * separate kernels), tile height tj (j) and run length seg (i) */
    int fused, stage_tj, stage_seg;
    /* tensor maps of the TMA-staged update (precision form, when the layout
     * allows it; else NULL) and how the split stage's update reads its inputs:
     * 0 thread loads, 1 TMA-staged tiles, 2 thread loads with an L2 prefetch
     * of the block one wave ahead */
    mhd::UpdMaps *maps;
    int upd_tma;
    mhd::StepScalars *d_sc, *h_sc;
    double *d_trig, *h_trig;
    float *d_trigf;
    mhd::MaxLoc *d_part, *h_part;
    int npart;
    int *d_cnt, *h_cnt;
    double *d_stage;             /* NSTAGE staging buffers of stage_n doubles (precision form) */
    long long stage_n;
    cudaStream_t st_cp[NSTAGE];  /* one copy stream per staging buffer */
    cudaEvent_t ev_cp[NSTAGE], ev_cvt[NSTAGE];
    std::vector<double> hx, hy, hz, hspL;
    double omdiff;
    int uploaded;
    cudaError_t last_cuda;
    /* mhd_run step graphs, one per starting primitive parity */
    cudaGraphExec_t gexecs[2];
    int graph_ready, graph_launches;
    int *d_cnt_run;
    /* instrumentation */
    long long launches;
    int prof, nslot;
    cudaEvent_t ev[2 * 256];
    int slot_kind[256];
    double prof_ms[MHD_PROF_NKIND];
    long long prof_n[MHD_PROF_NKIND];
    cudaEvent_t tev[2];
    /* asynchronous checkpoint: device snapshot, pinned host copy, writer */
    double *d_snap, *h_snap;
    cudaStream_t st_io;
    cudaEvent_t ev_snap, ev_host;
    std::thread writer;
    int ck_pending, ck_status;
};

/* batched form: one device-resident step of a context on a given stream
 * (mhd_ctx.cu) */
int mhd_ctx_prepare_run(mhd_ctx *ctx);
int mhd_ctx_enqueue_step(mhd_ctx *ctx, cudaStream_t s, long long *launches);

#endif
