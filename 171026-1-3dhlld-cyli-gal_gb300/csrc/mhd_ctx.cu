/*
 * mhd_ctx.cu -- the C-ABI of libmhdgpu.so (include/mhd_gpu.h): context
 * set-up, state transfer, and the step orchestration on one CUDA stream.
 *
 * Reference call chain replaced (main.c:316-393):
 *   Setdt()          -> mhd_setdt()          (setdt.h:24-94)
 *   SpiralGravity()  -> mhd_spiral_gravity() (spiralgravity.h:20-124)
 *   TVDRK()          -> mhd_tvdrk()          (tvdrungekutta.h:16-78)
 *
 * Device data layout: the reference's own, [m][i][j][k] with k fastest and one
 * ghost cell per side, so host<->device copies are plain memcpy.  The
 * j-independent grid tables (geometric factors, minimum cell length,
 * axisymmetric gravity) are stored once per (i,k).  Compiled with
 * --fmad=false (the gravity probe and the FP64 scalars must round as the
 * reference does).
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "mhd_ctx_internal.h"

using namespace mhd;



enum { PK_FLUX_R = 0, PK_FLUX_PHI = 1, PK_FLUX_Z = 2, PK_UPDATE = 3, PK_GHOST = 4, PK_SETDT = 5, PK_TRIG = 6,
       PK_CVT = 7, PK_STAGE = 8, PK_ZUPDATE = 9 };
static const int MAXSLOT = 256;

/* fold the recorded event pairs into the per-kind totals */
static cudaError_t prof_harvest(mhd_ctx *ctx)
{
    if (ctx->nslot == 0) return cudaSuccess;
    cudaError_t e = cudaEventSynchronize(ctx->ev[2 * ctx->nslot - 1]);
    if (e != cudaSuccess) return e;
    for (int s = 0; s < ctx->nslot; s++) {
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, ctx->ev[2 * s], ctx->ev[2 * s + 1]);
        if (e != cudaSuccess) return e;
        ctx->prof_ms[ctx->slot_kind[s]] += ms;
        ctx->prof_n[ctx->slot_kind[s]] += 1;
    }
    ctx->nslot = 0;
    return cudaSuccess;
}

static cudaError_t prof_begin(mhd_ctx *ctx, int kind)
{
    if (!ctx->prof) return cudaSuccess;
    if (ctx->nslot == MAXSLOT) {
        cudaError_t e = prof_harvest(ctx);
        if (e != cudaSuccess) return e;
    }
    ctx->slot_kind[ctx->nslot] = kind;
    return cudaEventRecord(ctx->ev[2 * ctx->nslot], ctx->st);
}

static cudaError_t prof_end(mhd_ctx *ctx)
{
    ctx->launches++;
    if (!ctx->prof) return cudaSuccess;
    cudaError_t e = cudaEventRecord(ctx->ev[2 * ctx->nslot + 1], ctx->st);
    ctx->nslot++;
    return e;
}

/* launch one kernel (the call returns its launch status) with optional timing */
#define LAUNCH(kind, call)            \
    do {                              \
        CK(prof_begin(ctx, kind));    \
        CK(call);                     \
        CK(prof_end(ctx));            \
    } while (0)

/* a failed call's error is returned and the runtime's last-error latch is
 * cleared, so the next launch check does not report it a second time */
#define CK(call)                                   \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) {                   \
            cudaGetLastError();                    \
            if (ctx) ctx->last_cuda = e_;          \
            return MHD_ERR_CUDA;                   \
        }                                          \
    } while (0)

static void *vcur_ptr(mhd_ctx *ctx) { return ctx->vcur == 0 ? ctx->Va : ctx->Vb; }
static void *vnext_ptr(mhd_ctx *ctx) { return ctx->vcur == 0 ? ctx->Vb : ctx->Va; }

/* ------------------------------------------------------------------------ */
/* small kernels that live here                                              */
/* ------------------------------------------------------------------------ */

/* cos/sin of the arm phase per (i,j) (spiralgravity.h:63-65) on the device,
 * for the precision form; the plain form fills the same table on the host
 * with the C library's sincos, the function the reference calls. */
__global__ void trig_kernel(int ixmax, int jymax, const double *__restrict__ y, const double *__restrict__ spL,
                            double armnum, double omdiff, const StepScalars *__restrict__ sc, double *trig,
                            float *trigf)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ixmax * jymax) return;
    int i = (int)(t / jymax), j = (int)(t % jymax);
    double phase = armnum * (y[j] - omdiff * sc->t + spL[i]);
    double s, c;
    sincos(phase, &s, &c);
    trig[t] = c;
    trig[(long long)ixmax * jymax + t] = s;
    trigf[t] = (float)c;
    trigf[(long long)ixmax * jymax + t] = (float)s;
}

__global__ void gravity_probe_kernel(Geom G, const StepScalars *__restrict__ sc, const double *__restrict__ trig,
                                     double *out)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G.nc) return;
    int k = (int)(t % G.kzmax);
    long long r = t / G.kzmax;
    int j = (int)(r % G.jymax), i = (int)(r / G.jymax);
    double gx, gy, gz;
    gravity_field(G, *sc, trig, i, j, k, gx, gy, gz);
    out[t] = gx;
    out[G.nc + t] = gy;
    out[2 * G.nc + t] = gz;
}

/* ------------------------------------------------------------------------ */
/* host helpers                                                              */
/* ------------------------------------------------------------------------ */
static int check_grid(const mhd_grid *g)
{
    if (!g || g->ix < 12 || g->kz < 12 || g->jy < 4 || (g->jy & 1)) return MHD_ERR_ARG;
    if (!g->x || !g->xm || !g->oneox || !g->oneodx || !g->y || !g->z || !g->oneodz || !g->dzm) return MHD_ERR_ARG;
    if (!g->g1 || !g->g2 || !g->g3 || !g->g4 || !g->g5 || !g->g6 || !g->minlength) return MHD_ERR_ARG;
    if (!g->x_absorb_factor || !g->z_absorb_factor || !g->c_absorb_factor) return MHD_ERR_ARG;
    if (g->irin < 0 || g->irin > g->ix) return MHD_ERR_ARG;
    return MHD_OK;
}

/* gather a j-independent table into [ni][nk]; returns MHD_ERR_ARG if a
 * reference-layout table actually varies with j over [j0, j1) */
static int gather_ik(const double *src, int compact, int ni, int nj, int nk, int j0, int j1, double *dst, int dst_nk)
{
    for (int i = 0; i < ni; i++)
        for (int k = 0; k < nk; k++) {
            double v;
            if (compact) v = src[(size_t)i * nk + k];
            else {
                v = src[((size_t)i * nj + j0) * nk + k];
                for (int j = j0 + 1; j < j1; j++)
                    if (memcmp(&src[((size_t)i * nj + j) * nk + k], &v, sizeof v) != 0) return MHD_ERR_ARG;
            }
            dst[(size_t)i * dst_nk + k] = v;
        }
    return MHD_OK;
}

static void free_all(mhd_ctx *ctx)
{
    if (ctx->writer.joinable()) ctx->writer.join();
    void *dev[] = {ctx->dtab, ctx->ftab, ctx->U, ctx->U1, ctx->Va, ctx->Vb, ctx->Uinit, ctx->Vinit,
                   ctx->rhofloor, ctx->F, ctx->Gf, ctx->H, ctx->Uraw, ctx->d_sc, ctx->d_trig, ctx->d_trigf,
                   ctx->d_part, ctx->d_cnt, ctx->d_stage, ctx->d_cnt_run, ctx->d_snap, ctx->Ulo, ctx->U1lo,
                   ctx->Urawlo, ctx->Zs, ctx->Hb};
    if (ctx->h_snap) cudaFreeHost(ctx->h_snap);
    for (int q = 0; q < NSTAGE; q++) {
        if (ctx->ev_cp[q]) cudaEventDestroy(ctx->ev_cp[q]);
        if (ctx->ev_cvt[q]) cudaEventDestroy(ctx->ev_cvt[q]);
        if (ctx->st_cp[q]) { cudaStreamSynchronize(ctx->st_cp[q]); cudaStreamDestroy(ctx->st_cp[q]); }
    }
    if (ctx->ev_snap) cudaEventDestroy(ctx->ev_snap);
    if (ctx->ev_host) cudaEventDestroy(ctx->ev_host);
    if (ctx->st_io) cudaStreamDestroy(ctx->st_io);
    for (size_t q = 0; q < sizeof dev / sizeof dev[0]; q++)
        if (dev[q]) cudaFree(dev[q]);
    if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
    if (ctx->h_trig) cudaFreeHost(ctx->h_trig);
    if (ctx->h_part) cudaFreeHost(ctx->h_part);
    if (ctx->h_cnt) cudaFreeHost(ctx->h_cnt);
    for (int q = 0; q < 2; q++)
        if (ctx->gexecs[q]) cudaGraphExecDestroy(ctx->gexecs[q]);
    for (int q = 0; q < 2 * MAXSLOT; q++)
        if (ctx->ev[q]) cudaEventDestroy(ctx->ev[q]);
    for (int q = 0; q < 2; q++)
        if (ctx->tev[q]) cudaEventDestroy(ctx->tev[q]);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    for (int q = 0; q < MHD_MAX_SLABS; q++)
        if (ctx->ev_slab[q]) cudaEventDestroy(ctx->ev_slab[q]);
    if (ctx->ev_upd) cudaEventDestroy(ctx->ev_upd);
    if (ctx->st_upd) { cudaStreamSynchronize(ctx->st_upd); cudaStreamDestroy(ctx->st_upd); }
    if (ctx->st_aux) { cudaStreamSynchronize(ctx->st_aux); cudaStreamDestroy(ctx->st_aux); }
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx->maps;
}

/* Tensor maps for the TMA-staged update: each FP32 array viewed as a 2D tensor
 * [nvar][nc] (row stride nc * 4 bytes, a multiple of 16 only when nc % 4 == 0;
 * tile coordinates are 32-bit).  cuTensorMapEncodeTiled comes from the driver
 * through the runtime's entry-point query, so the library links no driver
 * library.  NULL when the layout or the driver does not allow it. */
typedef CUresult (*encode_tiled_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static UpdMaps *make_upd_maps(mhd_ctx *ctx)
{
    if (!ctx->fp32 || ctx->nc % 4 != 0 || ctx->nc + 2 * MHD_UPD_TILE >= (1LL << 31)) return NULL;
    void *fn = NULL;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) != cudaSuccess ||
        qr != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return NULL;
    }
    encode_tiled_fn enc = (encode_tiled_fn)fn;
    UpdMaps *m = new (std::nothrow) UpdMaps;
    if (!m) return NULL;
    auto mk = [&](CUtensorMap *t, void *base, int nvar, int box) {
        cuuint64_t dims[2] = {(cuuint64_t)ctx->nc, (cuuint64_t)nvar};
        cuuint64_t strides[1] = {(cuuint64_t)ctx->nc * sizeof(float)};
        cuuint32_t boxd[2] = {(cuuint32_t)box, (cuuint32_t)nvar};
        cuuint32_t es[2] = {1, 1};
        return enc(t, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, boxd, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    const int T = MHD_UPD_TILE, W = MHD_UPD_WIDE;
    bool ok = mk(&m->v[0], ctx->Va, 9, T) && mk(&m->v[1], ctx->Vb, 9, T) && mk(&m->f, ctx->F, 9, T) &&
              mk(&m->g, ctx->Gf, 9, T) && mk(&m->un, ctx->U, 9, T) && mk(&m->u1, ctx->U1, 9, T) &&
              mk(&m->fm, ctx->F, 9, W) && mk(&m->gm, ctx->Gf, 9, W) && mk(&m->h, ctx->H, 9, W) &&
              mk(&m->rho, ctx->rhofloor, 1, T);
    if (!ok) {
        delete m;
        return NULL;
    }
    return m;
}

/* ------------------------------------------------------------------------ */
/* create / destroy                                                          */
/* ------------------------------------------------------------------------ */
extern "C" int mhd_create(const mhd_grid *g, const mhd_params *p, mhd_ctx **out)
{
    mhd_ctx *ctx = NULL;
    if (!out || !p) return MHD_ERR_ARG;
    *out = NULL;
    int rc = check_grid(g);
    if (rc) return rc;
    if (p->limiter < 0 || p->limiter > 3 || p->solver < 0 || p->solver > 1 || p->source < 0 || p->source > 3 ||
        (p->scheme != MHD_SCHEME_RK2 && p->scheme != MHD_SCHEME_RK3) || p->precision < 0 || p->precision > 2)
        return MHD_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return MHD_ERR_NODEV;

    ctx = new (std::nothrow) mhd_ctx();
    if (!ctx) return MHD_ERR_NOMEM;
    ctx->fused = 0;
    ctx->stage_tj = 7;
    ctx->stage_seg = 32;
    memset((void *)&ctx->G, 0, sizeof ctx->G);
    cudaGetDevice(&ctx->device);
    if (cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || ctx->nsm < 1) {
        cudaGetLastError();
        ctx->nsm = 152;
    }
    ctx->p = *p;
    ctx->ix = g->ix; ctx->jy = g->jy; ctx->kz = g->kz;
    ctx->ixmax = g->ix + 2; ctx->jymax = g->jy + 2; ctx->kzmax = g->kz + 2;
    ctx->irin = g->irin;
    ctx->nc = (long long)ctx->ixmax * ctx->jymax * ctx->kzmax;
    ctx->fp32 = p->precision == MHD_PREC_FP32 || p->precision == MHD_PREC_FP32X2;
    ctx->pair = p->precision == MHD_PREC_FP32X2;
    ctx->esz = ctx->fp32 ? sizeof(float) : sizeof(double);
    const int ixmax = ctx->ixmax, jymax = ctx->jymax, kzmax = ctx->kzmax;
    const long long nc = ctx->nc;

    /* ---- host tables ---- */
    const size_t nik = (size_t)ixmax * kzmax;
    std::vector<double> gtab(6 * nik, 0.0), minl(nik), grax(3 * nik, 0.0);
    const double *gsrc[6] = {g->g1, g->g2, g->g3, g->g4, g->g5, g->g6};
    for (int n = 0; n < 6; n++) {
        /* face-shaped [ixmax-1][jymax-1][kzmax-1]; rows j=0 are never read */
        rc = gather_ik(gsrc[n], g->compact, ixmax - 1, jymax - 1, kzmax - 1, 1, jymax - 1, &gtab[n * nik], kzmax);
        if (rc) { delete ctx; return rc; }
    }
    rc = gather_ik(g->minlength, g->compact, ixmax, jymax, kzmax, 0, jymax, minl.data(), kzmax);
    if (rc) { delete ctx; return rc; }
    const double *gr[3] = {g->Grxaxi, g->Gryaxi, g->Grzaxi};
    for (int n = 0; n < 3; n++)
        if (gr[n]) {
            rc = gather_ik(gr[n], g->compact, ixmax, jymax, kzmax, 0, jymax, &grax[n * nik], kzmax);
            if (rc) { delete ctx; return rc; }
        }

    /* spiral tables (spiralgravity.h:37-77), C-library math as the reference */
    const double a1 = 0.65, b1 = 0.026;
    double oneoscalephase = 1.0 / p->scalephase, oneoscaler = 1.0 / p->scaler;
    double cotpitch = 1.0 / tan(p->pitch);
    std::vector<double> spA(nik), spS(kzmax), spQ(kzmax), spR(kzmax), spC1(ixmax), spC2(ixmax), spD(ixmax),
        spL(ixmax);
    for (int i = 0; i < ixmax; i++) {
        double xi = g->x[i];
        double xoscalephase = xi * oneoscalephase;
        double xoscaler = xi * oneoscaler;
        double xoscaler2 = xoscaler * oneoscaler;
        double x2oscaler2 = xoscaler * xoscaler;
        double oneoonex2oscaler2 = 1.0 / (1.0 + x2oscaler2);
        double oneoonex2oscaler215 = 1.0 * pow(oneoonex2oscaler2, 1.5);
        spC1[i] = xoscaler2 * oneoonex2oscaler215;
        spC2[i] = x2oscaler2 * oneoonex2oscaler215;
        spD[i] = ((2.0 - x2oscaler2) * oneoonex2oscaler2);
        spL[i] = cotpitch * log(xoscalephase);
        double x2 = xi * xi;
        for (int k = 0; k < kzmax; k++) {
            double z2 = g->z[k] * g->z[k];
            double a1zk2b12 = ((a1 + sqrt(z2 + b1 * b1)) * (a1 + sqrt(z2 + b1 * b1)));
            spA[(size_t)i * kzmax + k] = 1.0 / sqrt(x2 + a1zk2b12);
        }
    }
    for (int k = 0; k < kzmax; k++) {
        double z2 = g->z[k] * g->z[k];
        spS[k] = (p->scalez / sqrt(z2 + p->scalez * p->scalez));
        spQ[k] = (1.0 + a1 / sqrt(z2 + b1 * b1));
        spR[k] = 1.0 / (z2 + p->scalez * p->scalez);
    }
    std::vector<double> dvol(nik, 0.0);
    for (int i = 1; i < ixmax - 1; i++)
        for (int k = 1; k < kzmax - 1; k++)
            dvol[(size_t)i * kzmax + k] = 0.5 * (g->xm[i] * g->xm[i] - g->xm[i - 1] * g->xm[i - 1]) * g->dy * g->dzm[k - 1];
    ctx->hx.assign(g->x, g->x + ixmax);
    ctx->hy.assign(g->y, g->y + jymax);
    ctx->hz.assign(g->z, g->z + kzmax);
    ctx->hspL = spL;
    ctx->omdiff = p->omegapattern - p->omegasp;

    /* ---- pack double tables ---- */
    std::vector<double> T;
    auto put = [&](const double *src, size_t n) { size_t off = T.size(); T.insert(T.end(), src, src + n); return off; };
    std::vector<double> oneodz(g->oneodz, g->oneodz + kzmax);
    size_t o_x = put(g->x, ixmax), o_xm = put(g->xm, ixmax), o_ox = put(g->oneox, ixmax);
    size_t o_odx = put(g->oneodx, ixmax), o_odz = put(oneodz.data(), kzmax);
    size_t o_g = put(gtab.data(), 6 * nik);
    size_t o_xabs = put(g->x_absorb_factor, 11), o_zabs = put(g->z_absorb_factor, 11);
    size_t o_cabs = put(g->c_absorb_factor, (size_t)(g->irin + 1) * kzmax);
    size_t o_minl = put(minl.data(), nik), o_grax = put(grax.data(), 3 * nik);
    size_t o_spA = put(spA.data(), nik), o_spS = put(spS.data(), kzmax), o_spQ = put(spQ.data(), kzmax);
    size_t o_spR = put(spR.data(), kzmax), o_C1 = put(spC1.data(), ixmax), o_C2 = put(spC2.data(), ixmax);
    size_t o_D = put(spD.data(), ixmax), o_L = put(spL.data(), ixmax), o_y = put(g->y, jymax);
    size_t o_z = put(g->z, kzmax);
    size_t o_dvol = put(dvol.data(), nik);
    std::vector<float> TF(T.begin(), T.end());   /* FP32 copies at the same offsets */
    const size_t o_oxlo = TF.size();              /* the low words of the FP32 1/x (pair-state form) */
    for (int i = 0; i < ixmax; i++) TF.push_back((float)(g->oneox[i] - (double)(float)g->oneox[i]));

#define CKC(call)                                  \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) {                   \
            cudaGetLastError();                    \
            free_all(ctx); delete ctx;             \
            return e_ == cudaErrorMemoryAllocation ? MHD_ERR_NOMEM : MHD_ERR_CUDA; \
        }                                          \
    } while (0)

    CKC(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking));
    CKC(cudaStreamCreateWithFlags(&ctx->st_aux, cudaStreamNonBlocking));
    CKC(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    CKC(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    CKC(ctx->fp32 ? prepare_stage((float *)0) : prepare_stage((double *)0));
    CKC(cudaMalloc((void **)&ctx->dtab, T.size() * sizeof(double)));
    CKC(cudaMalloc((void **)&ctx->ftab, TF.size() * sizeof(float)));
    CKC(cudaMemcpy(ctx->dtab, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice));
    CKC(cudaMemcpy(ctx->ftab, TF.data(), TF.size() * sizeof(float), cudaMemcpyHostToDevice));

    Geom &G = ctx->G;
    G.ixmax = ixmax; G.jymax = jymax; G.kzmax = kzmax; G.jy = g->jy; G.irin = g->irin; G.nc = nc;
    double *D = ctx->dtab;
    float *Fd = ctx->ftab;
    G.d.x = D + o_x; G.d.xm = D + o_xm; G.d.oneox = D + o_ox; G.d.oneodx = D + o_odx; G.d.oneodz = D + o_odz;
    G.d.g = D + o_g; G.d.xabs = D + o_xabs; G.d.zabs = D + o_zabs; G.d.cabs = D + o_cabs; G.d.oneody = g->oneody;
    G.f.x = Fd + o_x; G.f.xm = Fd + o_xm; G.f.oneox = Fd + o_ox; G.f.oneodx = Fd + o_odx; G.f.oneodz = Fd + o_odz;
    G.f.g = Fd + o_g; G.f.xabs = Fd + o_xabs; G.f.zabs = Fd + o_zabs; G.f.cabs = Fd + o_cabs;
    G.f.oneody = (float)g->oneody;
    G.d.minlength = D + o_minl; G.f.minlength = Fd + o_minl;
    G.minlength = D + o_minl; G.minminlength = g->minminlength; G.graxi = D + o_grax;
    G.spA = D + o_spA; G.spS = D + o_spS; G.spQ = D + o_spQ; G.spR = D + o_spR;
    G.spC1 = D + o_C1; G.spC2 = D + o_C2; G.spD = D + o_D; G.spL = D + o_L; G.y = D + o_y; G.z = D + o_z;
    G.dvol = D + o_dvol; G.dy = g->dy;
    G.oneoxlo = Fd + o_oxlo;
    G.graxif = Fd + o_grax; G.spAf = Fd + o_spA; G.spSf = Fd + o_spS; G.spQf = Fd + o_spQ; G.spRf = Fd + o_spR;
    G.spC1f = Fd + o_C1; G.spC2f = Fd + o_C2; G.spDf = Fd + o_D; G.zf = Fd + o_z;
    G.armnumf = (float)p->armnum; G.cotpitchf = (float)cotpitch;
    G.omegasp = p->omegasp; G.prcr = p->prcr; G.betacr = p->betacr; G.rhocr = p->rhocr;
    G.oneobetacr = 1.0 / p->betacr;
    G.omegaspf = (float)p->omegasp; G.prcrf = (float)p->prcr; G.betacrf = (float)p->betacr;
    G.oneobetacrf = (float)(1.0 / p->betacr);
    G.armnum = (double)p->armnum; G.cotpitch = cotpitch;
    G.cooling = p->cooling; G.gravity = p->gravity; G.limiter = p->limiter; G.solver = p->solver;
    G.scheme = p->scheme;
    G.source = p->source;
    G.repair_irmax = ctx->fp32 ? 4 : 0;

    /* ---- state ---- */
    size_t s9 = 9 * (size_t)nc * ctx->esz;
    void **bufs9[] = {&ctx->U, &ctx->U1, &ctx->Va, &ctx->Vb, &ctx->Uinit, &ctx->Vinit, &ctx->F, &ctx->Gf, &ctx->H,
                      &ctx->Uraw};
    for (size_t q = 0; q < sizeof bufs9 / sizeof bufs9[0]; q++) {
        CKC(cudaMalloc(bufs9[q], s9));
        CKC(cudaMemsetAsync(*bufs9[q], 0, s9, ctx->st));
    }
    CKC(cudaMalloc(&ctx->rhofloor, (size_t)nc * ctx->esz));
    CKC(cudaMalloc(&ctx->Zs, 18 * (size_t)(ixmax - 2) * (jymax - 2) * ctx->esz));
    CKC(cudaMalloc(&ctx->Hb, 9 * (size_t)(ixmax - 2) * (jymax - 2) * ctx->esz));
    if (ctx->pair) {
        float **lo9[] = {&ctx->Ulo, &ctx->U1lo, &ctx->Urawlo};
        for (int q = 0; q < 3; q++) {
            CKC(cudaMalloc((void **)lo9[q], s9));
            CKC(cudaMemsetAsync(*lo9[q], 0, s9, ctx->st));
        }
    }
    CKC(cudaMalloc((void **)&ctx->d_sc, sizeof(StepScalars)));
    CKC(cudaMallocHost((void **)&ctx->h_sc, sizeof(StepScalars)));
    memset(ctx->h_sc, 0, sizeof(StepScalars));
    CKC(cudaMemcpy(ctx->d_sc, ctx->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice));
    size_t ntrig = 2 * (size_t)ixmax * jymax;
    CKC(cudaMalloc((void **)&ctx->d_trig, ntrig * sizeof(double)));
    CKC(cudaMemset(ctx->d_trig, 0, ntrig * sizeof(double)));
    CKC(cudaMalloc((void **)&ctx->d_trigf, ntrig * sizeof(float)));
    CKC(cudaMemset(ctx->d_trigf, 0, ntrig * sizeof(float)));
    CKC(cudaMallocHost((void **)&ctx->h_trig, ntrig * sizeof(double)));
    long long ndt = (long long)(ixmax - 12) * (jymax - 2) * (kzmax - 2);
    ctx->npart = (int)((ndt + 255) / 256);
    if (ctx->npart > 2048) ctx->npart = 2048;
    if (ctx->npart < 1) ctx->npart = 1;
    CKC(cudaMalloc((void **)&ctx->d_part, ctx->npart * sizeof(MaxLoc)));
    CKC(cudaMallocHost((void **)&ctx->h_part, ctx->npart * sizeof(MaxLoc)));
    CKC(cudaMalloc((void **)&ctx->d_cnt, 3 * 3 * sizeof(int)));
    CKC(cudaMallocHost((void **)&ctx->h_cnt, 3 * 3 * sizeof(int)));
    ctx->maps = make_upd_maps(ctx);
    ctx->upd_tma = 0;
    ctx->stage_n = 1LL << 24;
    if (ctx->fp32) {
        CKC(cudaMalloc((void **)&ctx->d_stage, NSTAGE * ctx->stage_n * sizeof(double)));
        for (int q = 0; q < NSTAGE; q++) {
            CKC(cudaStreamCreateWithFlags(&ctx->st_cp[q], cudaStreamNonBlocking));
            CKC(cudaEventCreateWithFlags(&ctx->ev_cp[q], cudaEventDisableTiming));
            CKC(cudaEventCreateWithFlags(&ctx->ev_cvt[q], cudaEventDisableTiming));
        }
    }
    CKC(cudaStreamSynchronize(ctx->st));
#undef CKC
    *out = ctx;
    return MHD_OK;
}

extern "C" void mhd_destroy(mhd_ctx *ctx)
{
    if (!ctx) return;
    cudaStreamSynchronize(ctx->st);
    free_all(ctx);
    delete ctx;
}

extern "C" void *mhd_stream(mhd_ctx *ctx) { return ctx ? (void *)ctx->st : NULL; }

/* device selection for one-process-per-GPU launches: the ordinal is checked
 * against the visible device count before cudaSetDevice */
extern "C" int mhd_use_device(int ordinal)
{
    mhd_ctx *ctx = NULL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MHD_ERR_NODEV;
    }
    if (ordinal < 0 || ordinal >= ndev) return MHD_ERR_ARG;
    CK(cudaSetDevice(ordinal));
    return MHD_OK;
}

extern "C" int mhd_current_device(int *ordinal)
{
    mhd_ctx *ctx = NULL;
    if (!ordinal) return MHD_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MHD_ERR_NODEV;
    }
    CK(cudaGetDevice(ordinal));
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* transfers                                                                 */
/* ------------------------------------------------------------------------ */
/* host FP64 -> device state of the context's type; with lo (pair-state
 * form) each value is split into the nearest FP32 value and the rest */
static int put_state(mhd_ctx *ctx, void *dst, const double *src, long long n, float *lo = NULL)
{
    if (!ctx->fp32) {
        CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
        return MHD_OK;
    }
    /* NSTAGE staging buffers, each with its own copy stream, so several copy
     * engines move chunks at once while the context stream converts the ones
     * that have arrived; all ordering is by events */
    int b = 0;
    for (long long off = 0; off < n; off += ctx->stage_n, b = (b + 1) % NSTAGE) {
        long long m = n - off < ctx->stage_n ? n - off : ctx->stage_n;
        double *buf = ctx->d_stage + b * ctx->stage_n;
        CK(cudaStreamWaitEvent(ctx->st_cp[b], ctx->ev_cvt[b], 0));   /* the buffer's last reader is done */
        CK(cudaMemcpyAsync(buf, src + off, m * sizeof(double), cudaMemcpyHostToDevice, ctx->st_cp[b]));
        CK(cudaEventRecord(ctx->ev_cp[b], ctx->st_cp[b]));
        CK(cudaStreamWaitEvent(ctx->st, ctx->ev_cp[b], 0));
        if (lo) LAUNCH(PK_CVT, launch_cvt_pair(buf, (float *)dst + off, lo + off, m, ctx->st));
        else LAUNCH(PK_CVT, launch_cvt(buf, (float *)dst + off, m, ctx->st));
        CK(cudaEventRecord(ctx->ev_cvt[b], ctx->st));
    }
    return MHD_OK;
}

static int get_state(mhd_ctx *ctx, double *dst, const void *src, long long n, const float *lo = NULL)
{
    if (!ctx->fp32) {
        CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
        return MHD_OK;
    }
    /* conversions on the context stream feed NSTAGE buffers whose copies out
     * run on their own copy streams; the context stream then waits for all */
    int b = 0;
    for (long long off = 0; off < n; off += ctx->stage_n, b = (b + 1) % NSTAGE) {
        long long m = n - off < ctx->stage_n ? n - off : ctx->stage_n;
        double *buf = ctx->d_stage + b * ctx->stage_n;
        CK(cudaStreamWaitEvent(ctx->st, ctx->ev_cp[b], 0));      /* the buffer's last copy is done */
        if (lo) LAUNCH(PK_CVT, launch_cvt_pair_back((const float *)src + off, lo + off, buf, m, ctx->st));
        else LAUNCH(PK_CVT, launch_cvt_back((const float *)src + off, buf, m, ctx->st));
        CK(cudaEventRecord(ctx->ev_cvt[b], ctx->st));
        CK(cudaStreamWaitEvent(ctx->st_cp[b], ctx->ev_cvt[b], 0));
        CK(cudaMemcpyAsync(dst + off, buf, m * sizeof(double), cudaMemcpyDeviceToHost, ctx->st_cp[b]));
        CK(cudaEventRecord(ctx->ev_cp[b], ctx->st_cp[b]));
    }
    for (int q = 0; q < NSTAGE; q++) CK(cudaStreamWaitEvent(ctx->st, ctx->ev_cp[q], 0));
    return MHD_OK;
}

extern "C" int mhd_upload(mhd_ctx *ctx, const double *U, const double *V, const double *Uinit, const double *Vinit,
                          const double *rhofloor)
{
    if (!ctx || !U || !V) return MHD_ERR_ARG;
    long long n9 = 9 * ctx->nc;
    int rc;
    if ((rc = put_state(ctx, ctx->U, U, n9, ctx->Ulo))) return rc;
    ctx->vcur = 0;
    if ((rc = put_state(ctx, ctx->Va, V, n9))) return rc;
    if ((rc = put_state(ctx, ctx->Uinit, Uinit ? Uinit : U, n9))) return rc;
    if ((rc = put_state(ctx, ctx->Vinit, Vinit ? Vinit : V, n9))) return rc;
    std::vector<double> rf;
    if (!rhofloor) {   /* SaveInitial: rhofloor = U[0]*rhocr (saveinitial.h:40) */
        rf.resize(ctx->nc);
        for (long long q = 0; q < ctx->nc; q++) rf[q] = U[q] * ctx->p.rhocr;
        rhofloor = rf.data();
    }
    if ((rc = put_state(ctx, ctx->rhofloor, rhofloor, ctx->nc))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    ctx->uploaded = 1;
    return MHD_OK;
}

extern "C" int mhd_upload_state(mhd_ctx *ctx, const double *U, const double *V)
{
    if (!ctx || !U) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    int rc;
    if ((rc = put_state(ctx, ctx->U, U, 9 * ctx->nc, ctx->Ulo))) return rc;
    ctx->vcur = 0;
    if (V) {
        if ((rc = put_state(ctx, ctx->Va, V, 9 * ctx->nc))) return rc;
    } else if (ctx->pair) {
        LAUNCH(PK_CVT, launch_derive_v_pair(ctx->G, (const float *)ctx->U, ctx->Ulo, (float *)ctx->Va, ctx->st));
    } else if (ctx->fp32) {   /* V = UtoV(U) on the device */
        LAUNCH(PK_CVT, launch_derive_v(ctx->G, (const float *)ctx->U, (float *)ctx->Va, ctx->st));
    } else {
        LAUNCH(PK_CVT, launch_derive_v(ctx->G, (const double *)ctx->U, (double *)ctx->Va, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));   /* the caller's arrays are free again on return */
    return MHD_OK;
}

extern "C" int mhd_download(mhd_ctx *ctx, double *U, double *V)
{
    if (!ctx) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    int rc;
    if (U && (rc = get_state(ctx, U, ctx->U, 9 * ctx->nc, ctx->Ulo))) return rc;
    if (V && (rc = get_state(ctx, V, vcur_ptr(ctx), 9 * ctx->nc))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* Setdt                                                                     */
/* ------------------------------------------------------------------------ */
static MaxLoc better_host(MaxLoc a, MaxLoc b)
{
    if (b.q < 0) return a;
    if (a.q < 0) return b;
    if (b.v > a.v || (b.v == a.v && b.q < a.q)) return b;
    return a;
}

extern "C" int mhd_setdt(mhd_ctx *ctx, double *dt, double *ch, int ijk[3])
{
    if (!ctx || !dt || !ch) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    if (ctx->fp32) LAUNCH(PK_SETDT, launch_setdt(ctx->G, (const float *)vcur_ptr(ctx), ctx->d_part, ctx->npart, ctx->st));
    else LAUNCH(PK_SETDT, launch_setdt(ctx->G, (const double *)vcur_ptr(ctx), ctx->d_part, ctx->npart, ctx->st));
    CK(cudaMemcpyAsync(ctx->h_part, ctx->d_part, ctx->npart * sizeof(MaxLoc), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    MaxLoc best = {0.0, -1};
    for (int b = 0; b < ctx->npart; b++) best = better_host(best, ctx->h_part[b]);
    double oneocfldt = best.q >= 0 ? best.v : 0.0;
    /* setdt.h:84,89 */
    *dt = ctx->p.cfl / oneocfldt;
    *ch = ctx->G.minminlength * oneocfldt;
    if (ijk) {
        if (best.q < 0) { ijk[0] = ijk[1] = ijk[2] = -1; }
        else {
            ijk[2] = (int)(best.q % ctx->kzmax);
            ijk[1] = (int)((best.q / ctx->kzmax) % ctx->jymax);
            ijk[0] = (int)(best.q / ((long long)ctx->kzmax * ctx->jymax));
        }
    }
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* SpiralGravity                                                             */
/* ------------------------------------------------------------------------ */
extern "C" int mhd_spiral_gravity(mhd_ctx *ctx, double t)
{
    if (!ctx) return MHD_ERR_ARG;
    const mhd_params *p = &ctx->p;
    /* spiralgravity.h:41-42 */
    double switchfunc = (t - p->tausp) / fabs(t - p->tausp);
    double epssp = 0.5 * p->epssp0 * (t / p->tausp * (1.0 - switchfunc) + (1.0 + switchfunc));
    ctx->h_sc->epssp = epssp;
    ctx->h_sc->t = t;
    if (!p->gravity) return MHD_OK;
    const int ixmax = ctx->ixmax, jymax = ctx->jymax;
    if (!ctx->fp32) {
        /* spiralgravity.h:63-65 with the C library's sincos */
        CK(cudaStreamSynchronize(ctx->st));   /* h_trig may still feed a copy in flight */
        double armnum = (double)p->armnum;
        for (int i = 0; i < ixmax; i++)
            for (int j = 0; j < jymax; j++) {
                double phase = armnum * (ctx->hy[j] - ctx->omdiff * t + ctx->hspL[i]);
                double s, c;
                sincos(phase, &s, &c);
                ctx->h_trig[(size_t)i * jymax + j] = c;
                ctx->h_trig[(size_t)ixmax * jymax + (size_t)i * jymax + j] = s;
            }
        CK(cudaMemcpyAsync(ctx->d_trig, ctx->h_trig, 2 * (size_t)ixmax * jymax * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->st));
    } else {
        CK(cudaMemcpyAsync(ctx->d_sc, ctx->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
        long long n = (long long)ixmax * jymax;
        CK(prof_begin(ctx, PK_TRIG));
        trig_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->st>>>(ixmax, jymax, ctx->G.y, ctx->G.spL,
                                                                       (double)p->armnum, ctx->omdiff, ctx->d_sc,
                                                                       ctx->d_trig, ctx->d_trigf);
        CK(cudaGetLastError());
        CK(prof_end(ctx));
    }
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* TVDRK                                                                     */
/* ------------------------------------------------------------------------ */
static Box flux_box(const mhd_ctx *ctx, int dir)
{
    Box b;
    b.i0 = dir == 0 ? 0 : 1; b.i1 = ctx->ixmax - 1;
    b.j0 = dir == 1 ? 0 : 1; b.j1 = ctx->jymax - 1;
    b.k0 = dir == 2 ? 0 : 1; b.k1 = ctx->kzmax - 1;
    return b;
}

/* The split stage's face fluxes: r, phi, then the z row walk (every z face
 * but the last of each row, whose slots it leaves in the scratch Zs) and the
 * last z face of each row into the compact Hb -- and into H as well when the
 * TMA-staged update, which reads H directly, is selected (Hfull). */
template <typename T>
static int split_fluxes(mhd_ctx *ctx, const T *V, const T *Vinit, T *F, T *Gf, T *H, int Hfull)
{
    LAUNCH(PK_FLUX_R, launch_flux(0, ctx->G, V, Vinit, ctx->d_sc, F, flux_box(ctx, 0), false, ctx->st));
    LAUNCH(PK_FLUX_PHI, launch_flux(1, ctx->G, V, Vinit, ctx->d_sc, Gf, flux_box(ctx, 1), false, ctx->st));
    /* one profiling slot for both z launches: every z face */
    CK(prof_begin(ctx, PK_FLUX_Z));
    CK(launch_flux_zwalk(ctx->G, V, Vinit, ctx->d_sc, H, (T *)ctx->Zs, ctx->st));
    ctx->launches++;
    CK(launch_flux_zlast(ctx->G, Vinit, ctx->d_sc, H, (T *)ctx->Hb, (const T *)ctx->Zs, Hfull, ctx->st));
    CK(prof_end(ctx));
    return MHD_OK;
}

template <typename T>
static int run_stage(mhd_ctx *ctx, int kind, int last, int *counters)
{
    const T *V = (const T *)vcur_ptr(ctx);
    const T *Vinit = (const T *)ctx->Vinit;
    T *F = (T *)ctx->F, *Gf = (T *)ctx->Gf, *H = (T *)ctx->H;
    StageArgs<T> a;
    a.V = V; a.F = F; a.G = Gf; a.H = H;
    a.Un = (T *)ctx->U; a.U1 = (T *)ctx->U1;
    a.Uinit = (const T *)ctx->Uinit; a.rhofloor = (const T *)ctx->rhofloor;
    a.Vout = (T *)vnext_ptr(ctx); a.Uraw = (T *)ctx->Uraw;
    a.sc = ctx->d_sc; a.trig = ctx->d_trig; a.trigf = ctx->d_trigf; a.kind = kind; a.last = last; a.counters = counters;
    a.Vinit = Vinit;
    a.zghost = ctx->fused == 0 || ctx->fused == 3;   /* the split updates fill the interior columns' k-plane ghosts */
    /* path 2: each update block prefetches the block one wave ahead into L2
     * (8 resident blocks of 128 threads per SM in the precision form) */
    a.prefetch = (ctx->upd_tma & 2) ? 8 * ctx->nsm : 0;
    a.wfromu = (ctx->upd_tma & 4) ? 1 : 0;
    if (ctx->pair) {
        /* pair-state form: the split flux kernels of the FP32 form, then the
         * pair update and boundary fills */
        if constexpr (sizeof(T) == 4) {
            PairArgs pa;
            pa.Unlo = ctx->Ulo; pa.U1lo = ctx->U1lo; pa.Urawlo = ctx->Urawlo;
            a.Hb = (const T *)ctx->Hb;
            if (int rc = split_fluxes<T>(ctx, V, Vinit, F, Gf, H, 0)) return rc;
            LAUNCH(PK_UPDATE, launch_update_pair(ctx->G, a, pa, ctx->st));
            LAUNCH(PK_GHOST, launch_ghost_pair(ctx->G, a, pa, ctx->st));
            ctx->vcur ^= 1;
            return MHD_OK;
        } else {
            return MHD_ERR_STATE;
        }
    } else if (ctx->fused == 1) {
        LAUNCH(PK_STAGE, launch_stage(ctx->G, a, ctx->stage_tj, ctx->stage_seg, ctx->st));
    } else if (ctx->fused == 3) {
        /* the split kernels pipelined over ns slabs of i planes: the fluxes of
         * slab s on the context's stream, then its update on the update
         * stream, so the update of slab s (HBM-bound) runs beside the fluxes
         * of slab s+1 (issue-bound).  Slab s [a, b) needs the r faces a-1 ..
         * b-1; slab 0 computes faces 0 .. b-1 and slab s > 0 faces a .. b-1
         * (face a-1 is the slab before's), so every face is computed once and
         * the update of slab s waits only for the fluxes through slab s. */
        const int ni = ctx->ixmax - 2;
        const int ns = ctx->stage_seg < ni ? ctx->stage_seg : ni;
        CK(cudaEventRecord(ctx->ev_fork, ctx->st));
        CK(cudaStreamWaitEvent(ctx->st_upd, ctx->ev_fork, 0));
        for (int sl = 0; sl < ns; sl++) {
            const int a0 = 1 + (int)((long long)ni * sl / ns), b0 = 1 + (int)((long long)ni * (sl + 1) / ns);
            Box br = flux_box(ctx, 0), bp = flux_box(ctx, 1), bz = flux_box(ctx, 2);
            br.i0 = sl == 0 ? 0 : a0;
            br.i1 = b0;
            bp.i0 = bz.i0 = a0;
            bp.i1 = bz.i1 = b0;
            LAUNCH(PK_FLUX_R, launch_flux(0, ctx->G, V, Vinit, ctx->d_sc, F, br, false, ctx->st));
            LAUNCH(PK_FLUX_PHI, launch_flux(1, ctx->G, V, Vinit, ctx->d_sc, Gf, bp, false, ctx->st));
            CK(launch_zedge(ctx->G, V, Vinit, ctx->d_sc, H, bz, ctx->st));
            ctx->launches++;
            LAUNCH(PK_FLUX_Z, launch_flux_zinterior(ctx->G, V, Vinit, ctx->d_sc, H, bz, ctx->st));
            CK(cudaEventRecord(ctx->ev_slab[sl], ctx->st));
            CK(cudaStreamWaitEvent(ctx->st_upd, ctx->ev_slab[sl], 0));
            a.ibeg = a0;
            a.iend = b0;
            CK(launch_update(ctx->G, a, ctx->st_upd));
            ctx->launches++;
        }
        a.ibeg = 1;
        a.iend = 0;
        CK(cudaEventRecord(ctx->ev_upd, ctx->st_upd));
        CK(cudaStreamWaitEvent(ctx->st, ctx->ev_upd, 0));
    } else if (ctx->fused == 2) {
        LAUNCH(PK_FLUX_R, launch_flux(0, ctx->G, V, Vinit, ctx->d_sc, F, flux_box(ctx, 0), false, ctx->st));
        LAUNCH(PK_FLUX_PHI, launch_flux(1, ctx->G, V, Vinit, ctx->d_sc, Gf, flux_box(ctx, 1), false, ctx->st));
        LAUNCH(PK_ZUPDATE, launch_zupdate(ctx->G, a, ctx->st));
    } else {
        const int hfull = ctx->upd_tma == 1;   /* the TMA-staged update reads H alone */
        if (!hfull) a.Hb = (const T *)ctx->Hb;
        if (int rc = split_fluxes<T>(ctx, V, Vinit, F, Gf, H, hfull)) return rc;
        if (ctx->upd_tma == 1)
            LAUNCH(PK_UPDATE, launch_update_tma(ctx->G, a, *ctx->maps, ctx->vcur, &ctx->d_sc->err, ctx->st));
        else
            LAUNCH(PK_UPDATE, launch_update(ctx->G, a, ctx->st));
    }
    LAUNCH(PK_GHOST, launch_ghost(ctx->G, a, ctx->st));
    ctx->vcur ^= 1;
    return MHD_OK;
}

static int run_stages(mhd_ctx *ctx, int *d_cnt)
{
    static const int rk3[3][2] = {{0, 0}, {1, 0}, {2, 1}};
    static const int rk2[2][2] = {{0, 0}, {3, 1}};
    int ns = ctx->p.scheme == MHD_SCHEME_RK2 ? 2 : 3;
    for (int s = 0; s < ns; s++) {
        int kind = ns == 2 ? rk2[s][0] : rk3[s][0], last = ns == 2 ? rk2[s][1] : rk3[s][1];
        int rc = ctx->fp32 ? run_stage<float>(ctx, kind, last, d_cnt + 3 * s)
                           : run_stage<double>(ctx, kind, last, d_cnt + 3 * s);
        if (rc) return rc;
    }
    return MHD_OK;
}

extern "C" int mhd_tvdrk(mhd_ctx *ctx, double dt, double ch, int counters[3])
{
    if (!ctx) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    StepScalars *h = ctx->h_sc;
    h->dt = dt;
    h->ch = ch;
    /* tvdrungekutta.h:33-34 (RK3 factor 1/3, live RK2 factor 1/2) */
    h->psicoef = ctx->p.scheme == MHD_SCHEME_RK2 ? exp(-dt * ch * MHD_ONEOCR * 0.5)
                                                 : exp(-dt * ch * MHD_ONEOCR * MHD_ONEO3);
    h->dtf = (float)h->dt; h->chf = (float)h->ch; h->psif = (float)h->psicoef;
    h->psifl = (float)(h->psicoef - (double)h->psif);
    h->dtbad = 0;
    CK(cudaMemcpyAsync(ctx->d_sc, h, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(ctx->d_cnt, 0, 9 * sizeof(int), ctx->st));
    int rc = run_stages(ctx, ctx->d_cnt);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->h_cnt, ctx->d_cnt, 9 * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(&h->err, &ctx->d_sc->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (h->err) {   /* a staged tile's copies did not land: that tile was left as it was */
        h->err = 0;
        return MHD_ERR_TIMEOUT;
    }
    int last = ctx->p.scheme == MHD_SCHEME_RK2 ? 1 : 2;
    if (counters) for (int c = 0; c < 3; c++) counters[c] = ctx->h_cnt[3 * last + c];
    return MHD_OK;
}

extern "C" int mhd_step(mhd_ctx *ctx, double *t, double *dt, double *ch, int counters[3])
{
    if (!ctx || !t) return MHD_ERR_ARG;
    double dtv, chv;
    int rc = mhd_setdt(ctx, &dtv, &chv, NULL);
    if (rc) return rc;
    if (dt) *dt = dtv;
    if (ch) *ch = chv;
    if (isinf(dtv) || dtv < ctx->p.dtmin) return MHD_ERR_DT;   /* main.c:331 */
    if (ctx->p.gravity && (rc = mhd_spiral_gravity(ctx, *t))) return rc;
    if ((rc = mhd_tvdrk(ctx, dtv, chv, counters))) return rc;
    *t = *t + dtv;
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* probes                                                                    */
/* ------------------------------------------------------------------------ */
static Box full_face_box(const mhd_ctx *ctx)
{
    Box b = {0, ctx->ixmax - 1, 0, ctx->jymax - 1, 0, ctx->kzmax - 1};
    return b;
}

extern "C" int mhd_dbg_limiter(mhd_ctx *ctx, int dir, double dt, double *Vl, double *Vr)
{
    if (!ctx || dir < 0 || dir > 2 || !Vl || !Vr) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    ctx->h_sc->dt = dt;
    ctx->h_sc->psicoef = 1.0;
    ctx->h_sc->dtf = (float)dt; ctx->h_sc->psif = 1.0f;
    CK(cudaMemcpyAsync(ctx->d_sc, ctx->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
    long long nf = 9LL * (ctx->ixmax - 1) * (ctx->jymax - 1) * (ctx->kzmax - 1);
    CK(cudaMemsetAsync(ctx->F, 0, nf * ctx->esz, ctx->st));
    CK(cudaMemsetAsync(ctx->Gf, 0, nf * ctx->esz, ctx->st));
    if (ctx->fp32)
        CK(launch_states(dir, ctx->G, (const float *)vcur_ptr(ctx), (const float *)ctx->Vinit, ctx->d_sc,
                         (float *)ctx->F, (float *)ctx->Gf, full_face_box(ctx), ctx->st));
    else
        CK(launch_states(dir, ctx->G, (const double *)vcur_ptr(ctx), (const double *)ctx->Vinit, ctx->d_sc,
                         (double *)ctx->F, (double *)ctx->Gf, full_face_box(ctx), ctx->st));
    int rc;
    if ((rc = get_state(ctx, Vl, ctx->F, nf))) return rc;
    if ((rc = get_state(ctx, Vr, ctx->Gf, nf))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return MHD_OK;
}

extern "C" int mhd_dbg_flux(mhd_ctx *ctx, int dir, double dt, double ch, double *Fo)
{
    if (!ctx || dir < 0 || dir > 2 || !Fo) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    ctx->h_sc->dt = dt;
    ctx->h_sc->ch = ch;
    ctx->h_sc->psicoef = 1.0;
    ctx->h_sc->dtf = (float)dt; ctx->h_sc->chf = (float)ch; ctx->h_sc->psif = 1.0f;
    CK(cudaMemcpyAsync(ctx->d_sc, ctx->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
    long long nf = 9LL * (ctx->ixmax - 1) * (ctx->jymax - 1) * (ctx->kzmax - 1);
    CK(cudaMemsetAsync(ctx->F, 0, nf * ctx->esz, ctx->st));
    if (ctx->fp32)
        CK(launch_flux(dir, ctx->G, (const float *)vcur_ptr(ctx), (const float *)ctx->Vinit, ctx->d_sc,
                       (float *)ctx->F, full_face_box(ctx), true, ctx->st));
    else
        CK(launch_flux(dir, ctx->G, (const double *)vcur_ptr(ctx), (const double *)ctx->Vinit, ctx->d_sc,
                       (double *)ctx->F, full_face_box(ctx), true, ctx->st));
    int rc = get_state(ctx, Fo, ctx->F, nf);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return MHD_OK;
}

extern "C" int mhd_dbg_source(mhd_ctx *ctx, double *S)
{
    if (!ctx || !S) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    double *d_S = NULL;
    CK(cudaMemcpyAsync(ctx->d_sc, ctx->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMallocAsync((void **)&d_S, 9 * ctx->nc * sizeof(double), ctx->st));
    cudaError_t e = ctx->fp32 ? launch_source(ctx->G, (const float *)vcur_ptr(ctx), ctx->d_sc, ctx->d_trig,
                                              ctx->d_trigf, d_S, ctx->st)
                              : launch_source(ctx->G, (const double *)vcur_ptr(ctx), ctx->d_sc, ctx->d_trig,
                                              ctx->d_trigf, d_S, ctx->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(S, d_S, 9 * ctx->nc * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
    cudaFreeAsync(d_S, ctx->st);
    CK(e);
    CK(cudaStreamSynchronize(ctx->st));
    return MHD_OK;
}

extern "C" int mhd_dbg_gravity(mhd_ctx *ctx, double *gr)
{
    if (!ctx || !gr) return MHD_ERR_ARG;
    double *d_g = NULL;
    CK(cudaMemcpyAsync(ctx->d_sc, ctx->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMallocAsync((void **)&d_g, 3 * ctx->nc * sizeof(double), ctx->st));
    gravity_probe_kernel<<<(unsigned)((ctx->nc + 127) / 128), 128, 0, ctx->st>>>(ctx->G, ctx->d_sc, ctx->d_trig,
                                                                                  d_g);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(gr, d_g, 3 * ctx->nc * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
    cudaFreeAsync(d_g, ctx->st);
    CK(e);
    CK(cudaStreamSynchronize(ctx->st));
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* device-resident stepping (precision form)                                 */
/* ------------------------------------------------------------------------ */

/* Fold the CFL partials and set this step's scalars on the device:
 * setdt.h:84,89, the guard of main.c:331, the psi factor of
 * tvdrungekutta.h:33-34 and the spiral amplitude of spiralgravity.h:41-42. */
__global__ void step_scalars_kernel(const MaxLoc *__restrict__ part, int n, double cfl, double minminlength,
                                    double dtmin, double psifac, double tausp, double epssp0, StepScalars *sc)
{
    __shared__ MaxLoc sm[32];
    MaxLoc best = {0.0, -1};
    for (int b = threadIdx.x; b < n; b += blockDim.x) {
        MaxLoc o = part[b];
        if (o.q >= 0 && (best.q < 0 || o.v > best.v || (o.v == best.v && o.q < best.q))) best = o;
    }
    for (int o = 16; o > 0; o >>= 1) {
        MaxLoc x;
        x.v = __shfl_down_sync(0xffffffffu, best.v, o);
        x.q = __shfl_down_sync(0xffffffffu, best.q, o);
        if (x.q >= 0 && (best.q < 0 || x.v > best.v || (x.v == best.v && x.q < best.q))) best = x;
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
        MaxLoc x = sm[w];
        if (x.q >= 0 && (best.q < 0 || x.v > best.v || (x.v == best.v && x.q < best.q))) best = x;
    }
    if (sc->dtbad) return;   /* a fired guard freezes the state and t */
    double oneocfldt = best.q >= 0 ? best.v : 0.0;
    double dt = cfl / oneocfldt, ch = minminlength * oneocfldt;
    sc->oneocfldt = oneocfldt;
    sc->argmax = best.q;
    if (isinf(dt) || dt < dtmin) { sc->dtbad = 1; return; }
    double t = sc->t;
    double sw = (t - tausp) / fabs(t - tausp);
    sc->epssp = 0.5 * epssp0 * (t / tausp * (1.0 - sw) + (1.0 + sw));
    sc->dt = dt;
    sc->ch = ch;
    sc->psicoef = exp(-dt * ch * MHD_ONEOCR * psifac);
    sc->dtf = (float)dt;
    sc->chf = (float)ch;
    sc->psif = (float)sc->psicoef;
    sc->psifl = (float)(sc->psicoef - (double)sc->psif);
}

__global__ void advance_t_kernel(StepScalars *sc)
{
    if (!sc->dtbad) sc->t += sc->dt;
}

/* the launches of one whole step, device-resident */
static int enqueue_device_step(mhd_ctx *ctx)
{
    const mhd_params *p = &ctx->p;
    CK(launch_setdt(ctx->G, (const float *)vcur_ptr(ctx), ctx->d_part, ctx->npart, ctx->st));
    ctx->launches++;
    double psifac = p->scheme == MHD_SCHEME_RK2 ? 0.5 : MHD_ONEO3;
    step_scalars_kernel<<<1, 1024, 0, ctx->st>>>(ctx->d_part, ctx->npart, p->cfl, ctx->G.minminlength, p->dtmin,
                                                 psifac, p->tausp, p->epssp0, ctx->d_sc);
    CK(cudaGetLastError());
    ctx->launches++;
    if (p->gravity) {
        long long n = (long long)ctx->ixmax * ctx->jymax;
        trig_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->st>>>(ctx->ixmax, ctx->jymax, ctx->G.y,
                                                                       ctx->G.spL, (double)p->armnum,
                                                                       ctx->omdiff, ctx->d_sc, ctx->d_trig,
                                                                       ctx->d_trigf);
        CK(cudaGetLastError());
        ctx->launches++;
    }
    int rc = run_stages(ctx, ctx->d_cnt_run);
    if (rc) return rc;
    advance_t_kernel<<<1, 1, 0, ctx->st>>>(ctx->d_sc);
    CK(cudaGetLastError());
    ctx->launches++;
    return MHD_OK;
}

/* for the batched form: one device-resident step of ctx enqueued on stream s
 * (captured with the other discs' into one graph); launches counts the
 * kernels.  mhd_ctx_prepare_run() first, outside any capture. */
int mhd_ctx_prepare_run(mhd_ctx *ctx)
{
    if (!ctx->d_cnt_run) CK(cudaMalloc((void **)&ctx->d_cnt_run, 9 * sizeof(int)));
    return MHD_OK;
}

int mhd_ctx_enqueue_step(mhd_ctx *ctx, cudaStream_t s, long long *launches)
{
    if (!ctx->d_cnt_run || !ctx->fp32) return MHD_ERR_STATE;
    cudaStream_t st0 = ctx->st;
    int prof = ctx->prof;
    long long l0 = ctx->launches;
    ctx->st = s;
    ctx->prof = 0;
    int rc = enqueue_device_step(ctx);
    ctx->st = st0;
    ctx->prof = prof;
    if (launches) *launches += ctx->launches - l0;
    ctx->launches = l0;
    return rc;
}

extern "C" int mhd_run(mhd_ctx *ctx, int nsteps, double *t)
{
    if (!ctx || !t || nsteps < 0) return MHD_ERR_ARG;
    if (!ctx->fp32) return MHD_ERR_ARG;   /* plain form: host exp/sincos for bitwise parity */
    if (!ctx->uploaded) return MHD_ERR_STATE;
    if (!ctx->d_cnt_run) CK(cudaMalloc((void **)&ctx->d_cnt_run, 9 * sizeof(int)));
    StepScalars *h = ctx->h_sc;
    h->t = *t;
    h->dtbad = 0;
    CK(cudaMemcpyAsync(ctx->d_sc, h, sizeof(StepScalars), cudaMemcpyHostToDevice, ctx->st));
    /* the graph bakes in which primitive buffer is current: capture one per
     * starting parity (an odd stage count flips it every step) */
    int nst = ctx->p.scheme == MHD_SCHEME_RK2 ? 2 : 3;
    if (!ctx->graph_ready) {
        int prof = ctx->prof;
        ctx->prof = 0;
        int v0 = ctx->vcur;
        long long l0 = ctx->launches;
        for (int vs = 0; vs < 2; vs++) {
            cudaGraph_t graph;
            ctx->vcur = vs;
            CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_device_step(ctx);
            cudaError_t e = cudaStreamEndCapture(ctx->st, &graph);
            if (rc) { ctx->prof = prof; ctx->vcur = v0; return rc; }
            CK(e);
            CK(cudaGraphInstantiate(&ctx->gexecs[vs], graph, 0));
            cudaGraphDestroy(graph);
        }
        ctx->graph_launches = (int)((ctx->launches - l0) / 2);
        ctx->launches = l0;
        ctx->vcur = v0;
        ctx->prof = prof;
        ctx->graph_ready = 1;
    }
    for (int s = 0; s < nsteps; s++) {
        CK(cudaGraphLaunch(ctx->gexecs[ctx->vcur], ctx->st));
        ctx->vcur ^= (nst & 1);
        ctx->launches += ctx->graph_launches;
    }
    CK(cudaMemcpyAsync(h, ctx->d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    *t = h->t;
    if (h->err) {
        h->err = 0;
        return MHD_ERR_TIMEOUT;
    }
    return h->dtbad ? MHD_ERR_DT : MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* asynchronous checkpoint (BinaryOutput, output.h:1202-1414)                */
/* ------------------------------------------------------------------------ */
extern "C" int mhd_checkpoint_wait(mhd_ctx *ctx)
{
    if (!ctx) return MHD_ERR_ARG;
    if (ctx->writer.joinable()) ctx->writer.join();
    int rc = ctx->ck_pending ? ctx->ck_status : MHD_OK;
    ctx->ck_pending = 0;
    return rc;
}

extern "C" int mhd_checkpoint_begin(mhd_ctx *ctx, const char *root, int nout, double t)
{
    if (!ctx || !root || nout < 0) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    int rc = mhd_checkpoint_wait(ctx);
    if (rc) return rc;
    const size_t n = 9 * (size_t)ctx->nc;
    if (!ctx->d_snap) {
        CK(cudaMalloc((void **)&ctx->d_snap, n * sizeof(double)));
        cudaError_t e = cudaMallocHost((void **)&ctx->h_snap, n * sizeof(double));
        if (e != cudaSuccess) {
            cudaFree(ctx->d_snap);
            ctx->d_snap = NULL;
            ctx->h_snap = NULL;
            ctx->last_cuda = e;
            return MHD_ERR_NOMEM;
        }
        CK(cudaStreamCreateWithFlags(&ctx->st_io, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->ev_snap, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_host, cudaEventDisableTiming | cudaEventBlockingSync));
    }
    /* snapshot on the step stream (ordered after the steps enqueued so far) */
    if (ctx->fp32) LAUNCH(PK_CVT, launch_cvt_back((const float *)vcur_ptr(ctx), ctx->d_snap, (long long)n, ctx->st));
    else CK(cudaMemcpyAsync(ctx->d_snap, vcur_ptr(ctx), n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->st));
    CK(cudaEventRecord(ctx->ev_snap, ctx->st));
    /* device -> host on the I/O stream, beside the following steps */
    CK(cudaStreamWaitEvent(ctx->st_io, ctx->ev_snap, 0));
    CK(cudaMemcpyAsync(ctx->h_snap, ctx->d_snap, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st_io));
    CK(cudaEventRecord(ctx->ev_host, ctx->st_io));
    ctx->ck_pending = 1;
    ctx->ck_status = MHD_OK;
    std::string dir(root);
    ctx->writer = std::thread([ctx, dir, nout, t]() {
        cudaSetDevice(ctx->device);
        if (cudaEventSynchronize(ctx->ev_host) != cudaSuccess) { ctx->ck_status = MHD_ERR_CUDA; return; }
        ctx->ck_status = mhd_binary_output_arrays(dir.c_str(), nout, t, ctx->ix, ctx->jy, ctx->kz,
                                                  ctx->hx.data(), ctx->hy.data(), ctx->hz.data(), ctx->h_snap);
    });
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* diagnostics                                                               */
/* ------------------------------------------------------------------------ */
template <typename T>
__global__ void __launch_bounds__(256) diag_kernel(Geom G, const T *__restrict__ U, const T *__restrict__ Ulo,
                                                   double *part)
{
    __shared__ double sm[5][8];
    const int nj = G.jymax - 2, rows = (G.ixmax - 2) * nj;
    const long long nc = G.nc;
    double acc[4] = {0.0, 0.0, 0.0, 0.0}, dmax = 0.0;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int i = 1 + r / nj, j = 1 + r % nj;
        const double xi = G.d.x[i], xp = G.d.x[i + 1], xmn = G.d.x[i - 1];
        for (int k = 1 + threadIdx.x; k < G.kzmax - 1; k += blockDim.x) {
            const long long q = cidx(G, i, j, k);
            const double dv = G.dvol[(long long)i * G.kzmax + k];
            double u0 = U[q], u2 = U[2 * nc + q], u7 = U[7 * nc + q], u8 = U[8 * nc + q];
            if (Ulo) { u0 += Ulo[q]; u2 += Ulo[2 * nc + q]; u7 += Ulo[7 * nc + q]; u8 += Ulo[8 * nc + q]; }
            acc[0] += u0 * dv;
            acc[1] += u2 * dv;
            acc[2] += u7 * dv;
            acc[3] += fabs(u8) * dv;
            const long long si = (long long)G.jymax * G.kzmax, sj = G.kzmax;
            double divb = (xp * (double)U[4 * nc + q + si] - xmn * (double)U[4 * nc + q - si]) / (xi * (xp - xmn))
                          + ((double)U[5 * nc + q + sj] - (double)U[5 * nc + q - sj]) / (xi * 2.0 * G.dy)
                          + ((double)U[6 * nc + q + 1] - (double)U[6 * nc + q - 1]) / (G.z[k + 1] - G.z[k - 1]);
            dmax = fmax(dmax, fabs(divb));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int c = 0; c < 4; c++) acc[c] += __shfl_down_sync(0xffffffffu, acc[c], o);
        dmax = fmax(dmax, __shfl_down_sync(0xffffffffu, dmax, o));
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int c = 0; c < 4; c++) sm[c][w] = acc[c];
        sm[4][w] = dmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double out[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int v = 0; v < (int)(blockDim.x >> 5); v++) {
            for (int c = 0; c < 4; c++) out[c] += sm[c][v];
            out[4] = fmax(out[4], sm[4][v]);
        }
        for (int c = 0; c < 5; c++) part[blockIdx.x * 5 + c] = out[c];
    }
}

extern "C" int mhd_diagnostics(mhd_ctx *ctx, mhd_diag *d)
{
    if (!ctx || !d) return MHD_ERR_ARG;
    if (!ctx->uploaded) return MHD_ERR_STATE;
    const int nblk = 1024;
    double *dp = NULL;
    std::vector<double> hp(5 * nblk);
    CK(cudaMallocAsync((void **)&dp, 5 * nblk * sizeof(double), ctx->st));
    if (ctx->fp32) diag_kernel<float><<<nblk, 256, 0, ctx->st>>>(ctx->G, (const float *)ctx->U, ctx->Ulo, dp);
    else diag_kernel<double><<<nblk, 256, 0, ctx->st>>>(ctx->G, (const double *)ctx->U, NULL, dp);
    cudaError_t e = cudaGetLastError();
    ctx->launches++;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hp.data(), dp, 5 * nblk * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
    cudaFreeAsync(dp, ctx->st);
    CK(e);
    CK(cudaStreamSynchronize(ctx->st));
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nblk; b++) {
        for (int c = 0; c < 4; c++) s[c] += hp[5 * b + c];
        s[4] = fmax(s[4], hp[5 * b + 4]);
    }
    d->mass = s[0]; d->angmom = s[1]; d->energy = s[2]; d->psi = s[3]; d->maxdivb = s[4];
    return MHD_OK;
}

/* ------------------------------------------------------------------------ */
/* instrumentation                                                           */
/* ------------------------------------------------------------------------ */
extern "C" int mhd_prof_enable(mhd_ctx *ctx, int on)
{
    if (!ctx) return MHD_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->st));
    if (on && !ctx->ev[0])
        for (int q = 0; q < 2 * MAXSLOT; q++) CK(cudaEventCreate(&ctx->ev[q]));
    ctx->nslot = 0;
    for (int k = 0; k < MHD_PROF_NKIND; k++) { ctx->prof_ms[k] = 0.0; ctx->prof_n[k] = 0; }
    ctx->prof = on ? 1 : 0;
    return MHD_OK;
}

extern "C" int mhd_set_stage_shape(mhd_ctx *ctx, int fused, int tj, int seg)
{
    if (!ctx || fused < 0 || fused > 3 || seg < 1 || (fused != 3 && tj != 7) || (fused == 3 && seg > MHD_MAX_SLABS) ||
        (ctx->pair && fused != 0))
        return MHD_ERR_ARG;
    if (fused == 3 && !ctx->st_upd) {
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CK(cudaStreamCreateWithPriority(&ctx->st_upd, cudaStreamNonBlocking, hi));
        for (int q = 0; q < MHD_MAX_SLABS; q++) CK(cudaEventCreateWithFlags(&ctx->ev_slab[q], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_upd, cudaEventDisableTiming));
    }
    ctx->fused = fused;
    ctx->stage_tj = tj;
    ctx->stage_seg = seg;
    if (ctx->graph_ready) {
        /* the captured step graphs bake in the old shape */
        CK(cudaStreamSynchronize(ctx->st));
        for (int q = 0; q < 2; q++)
            if (ctx->gexecs[q]) { cudaGraphExecDestroy(ctx->gexecs[q]); ctx->gexecs[q] = NULL; }
        ctx->graph_ready = 0;
    }
    return MHD_OK;
}

extern "C" int mhd_set_update_path(mhd_ctx *ctx, int tma)
{
    if (!ctx || tma < 0 || tma > 6 || tma == 3 || tma == 5 || (tma == 1 && !ctx->maps) || (tma > 1 && !ctx->fp32) ||
        (ctx->pair && tma != 0))
        return MHD_ERR_ARG;
    ctx->upd_tma = tma;
    if (ctx->graph_ready) {
        CK(cudaStreamSynchronize(ctx->st));
        for (int q = 0; q < 2; q++)
            if (ctx->gexecs[q]) { cudaGraphExecDestroy(ctx->gexecs[q]); ctx->gexecs[q] = NULL; }
        ctx->graph_ready = 0;
    }
    return MHD_OK;
}

extern "C" int mhd_set_state_rounding(mhd_ctx *ctx, int on)
{
    if (!ctx || ctx->fp32 || on < 0 || on > 1) return MHD_ERR_ARG;
    ctx->G.round_state = on;
    return MHD_OK;
}

extern "C" int mhd_update_path(const mhd_ctx *ctx)
{
    if (!ctx) return MHD_ERR_ARG;
    return ctx->upd_tma;
}

extern "C" int mhd_prof_read(mhd_ctx *ctx, double *ms, long long *launches)
{
    if (!ctx) return MHD_ERR_ARG;
    CK(prof_harvest(ctx));
    for (int k = 0; k < MHD_PROF_NKIND; k++) {
        if (ms) ms[k] = ctx->prof_ms[k];
        if (launches) launches[k] = ctx->prof_n[k];
    }
    return MHD_OK;
}

extern "C" long long mhd_launch_count(const mhd_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int mhd_timer_start(mhd_ctx *ctx)
{
    if (!ctx) return MHD_ERR_ARG;
    if (!ctx->tev[0]) {
        CK(cudaEventCreate(&ctx->tev[0]));
        CK(cudaEventCreate(&ctx->tev[1]));
    }
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaEventRecord(ctx->tev[0], ctx->st));
    return MHD_OK;
}

extern "C" int mhd_timer_stop(mhd_ctx *ctx, double *ms)
{
    if (!ctx || !ms || !ctx->tev[0]) return MHD_ERR_ARG;
    CK(cudaEventRecord(ctx->tev[1], ctx->st));
    CK(cudaEventSynchronize(ctx->tev[1]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ctx->tev[0], ctx->tev[1]));
    *ms = f;
    return MHD_OK;
}

extern "C" int mhd_pin(void *ptr, size_t bytes, int on)
{
    mhd_ctx *ctx = NULL;
    if (!ptr || !bytes) return MHD_ERR_ARG;
    if (on) CK(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    else CK(cudaHostUnregister(ptr));
    return MHD_OK;
}
