/*
 * mhd_batch.cu -- many independent discs of uneven sizes and parameters.
 *
 * The reference has no batched driver: each disc is one run of main.c:316-393
 * with its own Setdt/SpiralGravity/TVDRK.  Here every disc keeps its own
 * context (state, tables, dt), and a step of ALL discs is:
 *
 *   CFL reduction   one launch over row tiles of every disc (per-disc partials)
 *   step scalars    one block per disc: its dt, ch, psi factor, spiral
 *                   amplitude and dt guard (setdt.h:84-89, main.c:331,
 *                   tvdrungekutta.h:33-34, spiralgravity.h:41-42)
 *   arm phase       cos/sin per (i,j) of every disc with gravity
 *   3 RK stages     ONE persistent launch per stage: blocks take work items
 *                   from a global queue ordered in waves -- the r, phi and z
 *                   flux items of slab w (a slab = sl planes in r) of every
 *                   disc, then the update items of slab w - lag -- and the
 *                   ghost items last.  An update item waits (bounded spin)
 *                   until the flux items of its slab and the slab below are
 *                   done, a ghost item until its disc's update items are.
 *                   Every item a block waits for was taken earlier by a
 *                   running block, so the waits end.  The items run the
 *                   single-disc kernels' code (marched r/phi faces, the
 *                   z walk, the update, the ghost fill).
 *   advance         t += dt per disc whose guard did not fire
 *
 * captured as one CUDA graph per primitive-buffer parity.  Slab depth (the r
 * extent of the items), queue lag and the register cap (launch bounds) are
 * chosen by mhd_batch_tune(), which times candidates on the live state and
 * restores it.  The halo is read through L1 from global memory, so its depth
 * is the stencil's (2 cells) for every slab depth.
 *
 * Two other modes are tuner candidates: phased (one launch per stage phase
 * over all discs) and the disc graph (each disc's own single-disc step, the
 * discs dealt to parallel stream branches of one graph), which is the fastest
 * on the 64-disc workload.
 *
 * Precision form only (FP32 + FP64 repair, the per-cell code of the
 * single-disc kernels); a batch of plain FP64 discs is stepped disc by disc
 * through mhd_step, each bit-identical to the reference.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <string.h>

#include <new>
#include <algorithm>
#include <vector>

#include "mhd_ctx_internal.h"
#include "mhd_kernels.cuh"

using namespace mhd;

namespace mhd_batch_k {

struct DiscDev {
    Geom G;
    float *U, *U1, *Va, *Vb, *Uinit, *Vinit, *rhofloor, *F, *Gf, *H, *Uraw;
    StepScalars *sc;
    double *trig;
    float *trigf;
    MaxLoc *part;
    int *counters;          /* [3 stages][3] */
    Box fbox[3], ubox;      /* flux face boxes per direction, interior box (phased mode) */
    int ndt;
    /* persistent stage: the disc cut into slabs of sl interior planes in r;
     * work items are laid out kx lanes along k by ky rows (kx * ky = 128) */
    int sl, ns, kx, ky, tk, tjr, nruns, nghost;
    int foff;               /* this disc's slab counters in the stage's readiness array */
    int stall;              /* test hook: slab 0 waits for one flux item more than exist */
    double cfl, minminlength, dtmin, psifac, tausp, epssp0, omdiff, armnum;
    int gravity;
};

/* Persistent-stage configurations the tuner times: slab depth in r planes
 * (the r extent of a work item and the unit of readiness), queue lag (slabs
 * of flux items enqueued ahead of an update slab), and the register cap: the
 * kernel instantiated for 5 or 4 resident blocks of 128 threads per SM (at
 * most 102 or 128 registers per thread). */
struct TileCfg {
    int sl, lag, minb;
};
static const TileCfg CANDIDATES[] = {{16, 1, 5}, {16, 2, 5}, {8, 1, 8}, {16, 1, 8},
                                     {32, 1, 5}, {16, 1, 4}, {16, 2, 4}, {8, 2, 4}};
static const int NCAND = sizeof(CANDIDATES) / sizeof(CANDIDATES[0]);
#define MHD_ZROWS 16    /* (i,j) rows of a z item: 4 per warp */
#define MHD_UPLANES 4   /* planes of an update item */
#define MHD_SPIN_LIMIT (1 << 24)

__device__ __forceinline__ void add_counts(int a, int b, int c, int *counters)
{
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0 && (a | b | c)) {
        if (a) atomicAdd(&counters[0], a);
        if (b) atomicAdd(&counters[1], b);
        if (c) atomicAdd(&counters[2], c);
    }
}

/* bounded wait until *flag >= target; false (and the error flag set) if the
 * limit runs out */
__device__ __forceinline__ bool wait_at_least(int *flag, int target, int *err, int limit)
{
    for (int it = 0; it < limit; it++) {
        if (atomicAdd(flag, 0) >= target) {
            __threadfence();
            return true;
        }
        if (atomicAdd(err, 0)) return false;
        __nanosleep(256);
    }
    atomicExch(err, 1);
    return false;
}

/* a block's copy of its disc's geometry: table pointers are then read from
 * shared memory instead of being kept in registers or reloaded from the
 * descriptor in global memory */
__device__ __forceinline__ void load_geom(Geom &sG, const Geom &G)
{
    const int *src = (const int *)&G;
    int *dst = (int *)&sG;
    for (int w = threadIdx.x; w < (int)(sizeof(Geom) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
}

/* item kinds of the persistent stage, and the item counts of slab s of a disc */
enum { IT_R = 0, IT_P = 1, IT_Z = 2, IT_U = 3, IT_G = 4 };

__host__ __device__ __forceinline__ int cdiv(int a, int b) { return (a + b - 1) / b; }

__host__ __device__ __forceinline__ void slab_items(const DiscDev &D, int s, int &nR, int &nP, int &nZ, int &nU)
{
    const int ni = D.G.ixmax - 2, nj = D.G.jymax - 2;
    const int planes = min(D.sl, ni - s * D.sl);
    nR = D.tjr * D.tk;                                    /* (j,k) line tiles, all faces of the slab */
    nP = cdiv(planes, D.ky) * D.tk * D.nruns;             /* (i,k) line tiles x runs of 16 phi faces */
    nZ = cdiv(planes * nj, MHD_ZROWS);                    /* (i,j) rows, 16 per item */
    nU = cdiv(planes, MHD_UPLANES) * D.tjr * D.tk;        /* cell tiles, MHD_UPLANES planes each */
}

/* The work items, each a function of its own (not inlined) so the kernel's
 * register allocation is not the union of all five paths.  Slab s covers the
 * interior planes [a0, b0). */
__device__ __forceinline__ void slab_planes(const Geom &G, const DiscDev &D, int slab, int &a0, int &b0)
{
    a0 = 1 + slab * D.sl;
    b0 = min(a0 + D.sl, G.ixmax - 1);
}

/* r faces of the slab (slab 0 also face 0) on one (j,k) line per thread */
__device__ __noinline__ void item_r(const Geom &G, const DiscDev &D, const float *V, int slab, int local)
{
    int a0, b0;
    slab_planes(G, D, slab, a0, b0);
    const int tx = threadIdx.x % D.kx, ty = threadIdx.x / D.kx;
    const int j = 1 + (local / D.tk) * D.ky + ty, k = 1 + (local % D.tk) * D.kx + tx;
    if (j <= G.jymax - 2 && k <= G.kzmax - 2) march_run<float, 0, false>(G, V, D.Vinit, D.sc, D.F, j, k, slab == 0 ? 0 : a0, b0);
}

/* a run of 16 phi faces on one (i,k) line per thread */
__device__ __noinline__ void item_p(const Geom &G, const DiscDev &D, const float *V, int slab, int local)
{
    int a0, b0;
    slab_planes(G, D, slab, a0, b0);
    const int tx = threadIdx.x % D.kx, ty = threadIdx.x / D.kx;
    const int run = local % D.nruns, rest = local / D.nruns;
    const int i = a0 + (rest / D.tk) * D.ky + ty, k = 1 + (rest % D.tk) * D.kx + tx;
    const int nf = G.jymax - 1;
    if (i < b0 && k <= G.kzmax - 2) march_run<float, 1, false>(G, V, D.Vinit, D.sc, D.Gf, i, k, 16 * run, min(16 * run + 16, nf));
}

/* MHD_ZROWS (i,j) rows: per row the two boundary z faces, then the walk */
__device__ __noinline__ void item_z(const Geom &G, const DiscDev &D, const float *V, int slab, int local)
{
    int a0, b0;
    slab_planes(G, D, slab, a0, b0);
    const int nj = G.jymax - 2, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int rr = 0; rr < MHD_ZROWS / 4; rr++) {
        const int row = local * MHD_ZROWS + w * (MHD_ZROWS / 4) + rr;
        if (row >= (b0 - a0) * nj) break;   /* warp-uniform */
        const int i = a0 + row / nj, j = 1 + row % nj;
        if (lane < 2) flux_face<float, 2, false>(G, V, D.Vinit, D.sc, D.H, i, j, lane == 0 ? 0 : G.kzmax - 2);
        zwalk_row<float, false>(G, V, D.sc, D.H, i, j, 1, G.kzmax - 2);
    }
}

/* update of MHD_UPLANES planes of a (j,k) tile */
__device__ __noinline__ void item_u(const Geom &G, const StageArgs<float> &a, const DiscDev &D, int slab, int local)
{
    int a0, b0;
    slab_planes(G, D, slab, a0, b0);
    const int tx = threadIdx.x % D.kx, ty = threadIdx.x / D.kx;
    const int tkk = local % D.tk, rest = local / D.tk;
    const int j = 1 + (rest % D.tjr) * D.ky + ty, k = 1 + tkk * D.kx + tx, tp = rest / D.tjr;
    int c0 = 0, c1 = 0, c2 = 0;
    if (j <= G.jymax - 2 && k <= G.kzmax - 2)
        for (int ii = 0; ii < MHD_UPLANES; ii++) {
            const int i = a0 + tp * MHD_UPLANES + ii;
            if (i >= b0) break;
            const int f = update_cell<float>(G, a, i, j, k);
            c0 += f & 1; c1 += (f >> 1) & 1; c2 += (f >> 2) & 1;
        }
    add_counts(c0, c1, c2, a.counters);
}

/* 128 ghost cells (the rim of the k planes, the i and j planes) */
__device__ __noinline__ void item_g(const Geom &G, const StageArgs<float> &a, int local)
{
    const unsigned g = (unsigned)local * 128u + threadIdx.x;
    int f = 0;
    if (g < ghost_count(G, 1)) f = ghost_cell<float>(G, a, g);
    add_counts(f & 1, (f >> 1) & 1, (f >> 2) & 1, a.counters);
}

/* One persistent launch per RK stage over all discs.  Blocks take work items
 * from a queue ordered in waves: the flux items (r, phi, z) of slab w of every
 * disc, then the update items of slab w - lag.  An update item of slab s
 * waits -- a bounded spin, then the error flag -- until every flux item of
 * slabs s and s-1 of its disc is done (its lower r face belongs to slab s-1),
 * a ghost item until every update item of its disc is.  Everything an item
 * waits for sits earlier in the queue and was taken by a block already
 * running, so the waits end.  The items run the single-disc kernels' code:
 * march_run (r and phi faces, each cell reconstructed once per direction),
 * zwalk_row plus the two boundary z faces, update_cell, ghost_cell. */
template <int MINB>
__global__ void __launch_bounds__(128, MINB)
batch_pstage_kernel(const DiscDev *__restrict__ discs, const uint2 *__restrict__ items, int nitems, int *head,
                    int *fdone, int *udone, int *err, int spin, int kind, int last, int parity, int stage)
{
    __shared__ int s_t, s_ok, s_d;
    __shared__ Geom sG;
    __shared__ StageArgs<float> sA;   /* an update or ghost item's arguments, read from shared memory */
    if (threadIdx.x == 0) s_d = -1;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_t = atomicAdd(head, 1);
        __syncthreads();
        const int t = s_t;
        if (t >= nitems) return;
        const uint2 e = items[t];
        const int d = (int)e.x, type = (int)(e.y >> 28), slab = (int)((e.y >> 18) & 0x3ffu),
                  local = (int)(e.y & 0x3ffffu);
        const DiscDev &D = discs[d];
        if (s_d != d) {   /* block-uniform */
            __syncthreads();
            const int *src = (const int *)&D.G;
            int *dst = (int *)&sG;
            for (int w = tid; w < (int)(sizeof(Geom) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
            __syncthreads();
            if (tid == 0) s_d = d;
        }
        if (tid == 0) {
            int ok = 1;
            if (type == IT_U) {
                int nR, nP, nZ, nU;
                slab_items(D, slab, nR, nP, nZ, nU);
                ok = wait_at_least(&fdone[D.foff + slab], nR + nP + nZ + (slab == 0 ? D.stall : 0), err, spin);
                if (ok && slab > 0) {
                    slab_items(D, slab - 1, nR, nP, nZ, nU);
                    ok = wait_at_least(&fdone[D.foff + slab - 1], nR + nP + nZ + (slab == 1 ? D.stall : 0), err, spin);
                }
            } else if (type == IT_G) {
                int tot = 0;
                for (int q = 0; q < D.ns; q++) {
                    int nR, nP, nZ, nU;
                    slab_items(D, q, nR, nP, nZ, nU);
                    tot += nU;
                }
                ok = wait_at_least(&udone[d], tot, err, spin);
            }
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;
        const bool live = !D.sc->dtbad;
        const float *V = parity ? D.Vb : D.Va;
        if (live && type == IT_R) item_r(sG, D, V, slab, local);
        else if (live && type == IT_P) item_p(sG, D, V, slab, local);
        else if (live && type == IT_Z) item_z(sG, D, V, slab, local);
        else if (live) {
            if (tid == 0) {
                StageArgs<float> a;
                a.V = V; a.F = D.F; a.G = D.Gf; a.H = D.H; a.Un = D.U; a.U1 = D.U1;
                a.Uinit = D.Uinit; a.rhofloor = D.rhofloor; a.Vout = parity ? D.Va : D.Vb; a.Uraw = D.Uraw;
                a.Vinit = D.Vinit; a.sc = D.sc; a.trig = D.trig; a.trigf = D.trigf; a.kind = kind; a.last = last;
                a.counters = D.counters + 3 * stage;
                a.zghost = 1;   /* the update fills the interior columns' k-plane ghosts, the ghost items the rest */
                sA = a;
            }
            __syncthreads();
            if (type == IT_U) item_u(sG, sA, D, slab, local);
            else item_g(sG, sA, local);
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            if (type <= IT_Z) atomicAdd(&fdone[D.foff + slab], 1);
            else if (type == IT_U) atomicAdd(&udone[d], 1);
        }
    }
}

/* CFL reduction over row tiles of every disc: precision-form screening of
 * setdt_kernel (FP32 cells, FP64 re-evaluation of each tile's winner) */
__global__ void __launch_bounds__(256)
batch_setdt_kernel(const DiscDev *__restrict__ discs, const uint2 *__restrict__ tiles, int rows_per_tile)
{
    __shared__ MaxLoc sm[8];
    const uint2 e = tiles[blockIdx.x];
    const DiscDev &D = discs[e.x];
    const Geom &G = D.G;
    const float *V = (const float *)(e.y >> 31 ? D.Vb : D.Va);
    const int local = (int)(e.y & 0x7fffffffu);
    const int nj = G.jymax - 2, rows = (G.ixmax - 12) * nj;
    MaxLoc best = {0.0, -1};
    for (int r = local * rows_per_tile; r < (local + 1) * rows_per_tile && r < rows; r++) {
        const int i = 1 + r / nj, j = 1 + r % nj;
        for (int k = 1 + threadIdx.x; k < G.kzmax - 1; k += blockDim.x) {
            const long long q = cidx(G, i, j, k), nc = G.nc;
            float v0 = V[q], v1 = V[nc + q], v2v = V[2 * nc + q], v3 = V[3 * nc + q];
            float v4 = V[4 * nc + q], v5 = V[5 * nc + q], v6 = V[6 * nc + q], v7 = V[7 * nc + q];
            float v2 = v1 * v1 + v2v * v2v + v3 * v3;
            float b2 = v4 * v4 + v5 * v5 + v6 * v6;
            float t1 = sqrtf(v2 + ((float)MHD_GM * v7 + b2) / v0) / G.f.minlength[(long long)i * G.kzmax + k];
            int cl = G.cooling ? cooling_rate_f(v0, v7) : 0;
            float tc = (2.0f * ((v0 * v0 * (float)cl) / (1.5f * v7)));
            double tmp = (t1 != t1 || tc != tc) ? (double)INFINITY : (double)rmax<float>(t1, tc);
            if (tmp > best.v && tmp > 0.0) { best.v = tmp; best.q = q; }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        MaxLoc other;
        other.v = __shfl_down_sync(0xffffffffu, best.v, o);
        other.q = __shfl_down_sync(0xffffffffu, best.q, o);
        best = better(best, other);
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        MaxLoc b = sm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = better(b, sm[w]);
        if (b.q >= 0) {
            const int k = (int)(b.q % G.kzmax), i = (int)(b.q / ((long long)G.kzmax * G.jymax));
            b.v = cfl_rate64_strict<float>(G, V, i, b.q, k);
        }
        D.part[local] = b;
    }
}

/* one block per disc: fold its partials, set its step scalars */
__global__ void batch_scalars_kernel(const DiscDev *__restrict__ discs)
{
    __shared__ MaxLoc sm[32];
    const DiscDev &D = discs[blockIdx.x];
    MaxLoc best = {0.0, -1};
    for (int b = threadIdx.x; b < D.ndt; b += blockDim.x) best = better(best, D.part[b]);
    for (int o = 16; o > 0; o >>= 1) {
        MaxLoc x;
        x.v = __shfl_down_sync(0xffffffffu, best.v, o);
        x.q = __shfl_down_sync(0xffffffffu, best.q, o);
        best = better(best, x);
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = better(best, sm[w]);
    StepScalars *sc = D.sc;
    if (sc->dtbad) return;
    double oneocfldt = best.q >= 0 ? best.v : 0.0;
    double dt = D.cfl / oneocfldt, ch = D.minminlength * oneocfldt;
    sc->oneocfldt = oneocfldt;
    sc->argmax = best.q;
    if (isinf(dt) || dt < D.dtmin) { sc->dtbad = 1; return; }
    double t = sc->t;
    double sw = (t - D.tausp) / fabs(t - D.tausp);
    sc->epssp = 0.5 * D.epssp0 * (t / D.tausp * (1.0 - sw) + (1.0 + sw));
    sc->dt = dt;
    sc->ch = ch;
    sc->psicoef = exp(-dt * ch * MHD_ONEOCR * D.psifac);
    sc->dtf = (float)dt;
    sc->chf = (float)ch;
    sc->psif = (float)sc->psicoef;
}

__global__ void batch_trig_kernel(const DiscDev *__restrict__ discs)
{
    const DiscDev &D = discs[blockIdx.y];
    if (!D.gravity || D.sc->dtbad) return;
    const Geom &G = D.G;
    const int n = G.ixmax * G.jymax;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        int i = q / G.jymax, j = q % G.jymax;
        double phase = D.armnum * (G.y[j] - D.omdiff * D.sc->t + G.spL[i]);
        double s, c;
        sincos(phase, &s, &c);
        D.trig[q] = c;
        D.trig[n + q] = s;
        D.trigf[q] = (float)c;
        D.trigf[n + q] = (float)s;
    }
}

__global__ void batch_advance_kernel(const DiscDev *__restrict__ discs, int ndisc)
{
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < ndisc && !discs[d].sc->dtbad) discs[d].sc->t += discs[d].sc->dt;
}

/* Phased mode: one specialised launch per phase over the tiles of every disc;
 * stream order replaces the queue's waits.  A tile is 128 cells: by rows of
 * j times bx cells along k, bx = the disc's k extent rounded up to a warp
 * (at most 128). */
__device__ __forceinline__ bool cell_of_tile(const uint4 e, const Box &b, int &i, int &j, int &k)
{
    const int bx = (int)(e.w >> 20), k0 = (int)(e.w & 0xfffffu);
    i = (int)e.y;
    j = (int)e.z + (int)threadIdx.x / bx;
    k = k0 + (int)threadIdx.x % bx;
    return (int)threadIdx.x < 128 / bx * bx && k < b.k1 && j < b.j1;
}

template <int DIR>
__global__ void __launch_bounds__(128) batch_flux_kernel(const DiscDev *__restrict__ discs,
                                                         const uint4 *__restrict__ tiles, int parity)
{
    __shared__ Geom sG;
    const uint4 e = tiles[blockIdx.x];
    const DiscDev &D = discs[e.x];
    load_geom(sG, D.G);
    if (D.sc->dtbad) return;
    int i, j, k;
    if (!cell_of_tile(e, D.fbox[DIR], i, j, k)) return;
    float *Fd = DIR == 0 ? D.F : DIR == 1 ? D.Gf : D.H;
    flux_face<float, DIR, false>(sG, parity ? D.Vb : D.Va, D.Vinit, D.sc, Fd, i, j, k);
}

__device__ __forceinline__ StageArgs<float> stage_args(const DiscDev &D, int kind, int last, int parity, int stage)
{
    StageArgs<float> a;
    a.V = parity ? D.Vb : D.Va; a.F = D.F; a.G = D.Gf; a.H = D.H; a.Un = D.U; a.U1 = D.U1;
    a.Uinit = D.Uinit; a.rhofloor = D.rhofloor; a.Vout = parity ? D.Va : D.Vb; a.Uraw = D.Uraw; a.Vinit = D.Vinit;
    a.sc = D.sc; a.trig = D.trig; a.trigf = D.trigf; a.kind = kind; a.last = last;
    a.counters = D.counters + 3 * stage;
    return a;
}

__global__ void __launch_bounds__(128) batch_update_kernel(const DiscDev *__restrict__ discs,
                                                           const uint4 *__restrict__ tiles, int kind, int last,
                                                           int parity, int stage)
{
    __shared__ Geom sG;
    const uint4 e = tiles[blockIdx.x];
    const DiscDev &D = discs[e.x];
    load_geom(sG, D.G);
    if (D.sc->dtbad) return;
    StageArgs<float> a = stage_args(D, kind, last, parity, stage);
    int i, j, k, f = 0;
    if (cell_of_tile(e, D.ubox, i, j, k)) f = update_cell<float>(sG, a, i, j, k);
    add_counters(f, a.counters);
}

__global__ void __launch_bounds__(128) batch_ghost_kernel(const DiscDev *__restrict__ discs,
                                                          const uint2 *__restrict__ tiles, int kind, int last,
                                                          int parity, int stage)
{
    __shared__ Geom sG;
    const uint2 e = tiles[blockIdx.x];
    const DiscDev &D = discs[e.x];
    load_geom(sG, D.G);
    if (D.sc->dtbad) return;
    StageArgs<float> a = stage_args(D, kind, last, parity, stage);
    const unsigned g = e.y * blockDim.x + threadIdx.x;
    int f = 0;
    if (g < ghost_count(sG)) f = ghost_cell<float>(sG, a, g);
    add_counters(f, a.counters);
}

}  /* namespace mhd_batch_k */

using namespace mhd_batch_k;

struct mhd_batch {
    int n, persistent, nst;
    cudaStream_t st;
    std::vector<mhd_ctx *> ctx;
    std::vector<int> stopped;
    std::vector<DiscDev> hd;
    DiscDev *dd;
    TileCfg cfg;
    int nblk_stage;
    /* work items of the persistent stage, in queue order, and the CFL row tiles */
    uint2 *dtiles, *ddt;
    int ntiles, ndt_tiles, rows_per_tile;
    int nslabs;                 /* slab counters of all discs (readiness array length) */
    int qlen;                   /* ints per stage in dqueue: head, slab counters, per-disc update counts */
    int phased;                 /* 1: one launch per phase, 0: one persistent launch per stage */
    int discgraph;              /* 1: every disc's own device-resident step, all in one graph */
    int nbranch;                /*    on this many parallel stream branches */
    std::vector<cudaStream_t> bst;
    std::vector<cudaEvent_t> bev;
    long long step_launches;    /* kernels per step of the captured graph */
    uint4 *dph[4];              /* phased row tiles: flux r, phi, z, update */
    int nph[4];
    uint2 *dghost;
    int nghost_tiles;
    int *dqueue;    /* [3 stages][qlen] */
    int *derr;
    int *dcnt;      /* per disc [3][3] */
    cudaGraphExec_t gx[2];
    int graph_ready, parity;
    long long launches;
    int spin_limit;             /* iterations of a bounded device-side wait */
    int stall_disc;             /* test hook: this disc's flux count is never reached (-1: none) */
};

#define BCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) { cudaGetLastError(); return e_ == cudaErrorMemoryAllocation ? MHD_ERR_NOMEM : MHD_ERR_CUDA; } \
    } while (0)

static int ceil_div(int a, int b) { return (a + b - 1) / b; }

/* the persistent stage's work items for a configuration, in queue order */
static int build_tiles(mhd_batch *b, TileCfg c)
{
    const int n = b->n;
    int foff = 0, maxns = 0;
    for (int d = 0; d < n; d++) {
        DiscDev &D = b->hd[d];
        const int ni = D.G.ixmax - 2, nj = D.G.jymax - 2, nk = D.G.kzmax - 2;
        D.sl = c.sl;
        D.ns = cdiv(ni, c.sl);
        D.kx = 32 * cdiv(nk < 128 ? nk : 128, 32);
        if (D.kx == 96) D.kx = 128;   /* kx * ky = 128 */
        D.ky = 128 / D.kx;
        D.tk = cdiv(nk, D.kx);
        D.tjr = cdiv(nj, D.ky);
        D.nruns = cdiv(nj + 1, 16);
        D.nghost = cdiv((int)ghost_count(D.G, 1), 128);
        D.foff = foff;
        D.stall = d == b->stall_disc ? 1 : 0;
        foff += D.ns;
        maxns = std::max(maxns, D.ns);
    }
    std::vector<uint2> tl;
    auto push = [&](int d, int type, int slab, int cnt) {
        for (int l = 0; l < cnt; l++)
            tl.push_back(make_uint2(d, ((unsigned)type << 28) | ((unsigned)slab << 18) | (unsigned)l));
    };
    /* within a wave, all discs' items of one kind together: the blocks then
     * run one item kind at a time (the ncu capture of the kernel with the
     * kinds interleaved per disc showed 3.6 instruction-fetch stalls per
     * issued instruction) */
    for (int w = 0; w < maxns + c.lag; w++) {
        for (int type = IT_R; type <= IT_Z; type++)
            for (int d = 0; d < n; d++) {
                const DiscDev &D = b->hd[d];
                if (w >= D.ns) continue;
                int nR, nP, nZ, nU;
                slab_items(D, w, nR, nP, nZ, nU);
                push(d, type, w, type == IT_R ? nR : type == IT_P ? nP : nZ);
            }
        const int u = w - c.lag;
        for (int d = 0; d < n && u >= 0; d++) {
            const DiscDev &D = b->hd[d];
            if (u >= D.ns) continue;
            int nR, nP, nZ, nU;
            slab_items(D, u, nR, nP, nZ, nU);
            push(d, IT_U, u, nU);
        }
    }
    for (int d = 0; d < n; d++) push(d, IT_G, 0, b->hd[d].nghost);
    if (b->dtiles) cudaFree(b->dtiles);
    b->dtiles = NULL;
    b->ntiles = (int)tl.size();
    BCK(cudaMalloc((void **)&b->dtiles, tl.size() * sizeof(uint2)));
    BCK(cudaMemcpy(b->dtiles, tl.data(), tl.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    b->nslabs = foff;
    const int qlen = 1 + foff + n;
    if (qlen != b->qlen) {
        if (b->dqueue) cudaFree(b->dqueue);
        b->dqueue = NULL;
        BCK(cudaMalloc((void **)&b->dqueue, 3 * (size_t)qlen * sizeof(int)));
        b->qlen = qlen;
    }
    BCK(cudaMemcpy(b->dd, b->hd.data(), n * sizeof(DiscDev), cudaMemcpyHostToDevice));
    b->cfg = c;
    return MHD_OK;
}

static int stage_blocks(TileCfg c)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (c.minb == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_pstage_kernel<4>, 128, 0);
    else if (c.minb == 8) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_pstage_kernel<8>, 128, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_pstage_kernel<5>, 128, 0);
    if (per < 1) per = 1;
    return sms * per;
}

static cudaError_t launch_stage(mhd_batch *b, int *q, int kind, int last, int parity, int stage)
{
    const int nb = b->nblk_stage;
    int *head = q, *fdone = q + 1, *udone = q + 1 + b->nslabs;
    if (b->cfg.minb == 4)
        batch_pstage_kernel<4><<<nb, 128, 0, b->st>>>(b->dd, b->dtiles, b->ntiles, head, fdone, udone, b->derr,
                                                      b->spin_limit, kind, last, parity, stage);
    else if (b->cfg.minb == 8)
        batch_pstage_kernel<8><<<nb, 128, 0, b->st>>>(b->dd, b->dtiles, b->ntiles, head, fdone, udone, b->derr,
                                                      b->spin_limit, kind, last, parity, stage);
    else
        batch_pstage_kernel<5><<<nb, 128, 0, b->st>>>(b->dd, b->dtiles, b->ntiles, head, fdone, udone, b->derr,
                                                      b->spin_limit, kind, last, parity, stage);
    return cudaGetLastError();
}

/* the launches of one step of all discs, starting at primitive parity `parity` */
/* disc-graph mode: fork from the batch stream into nbranch streams, each
 * running its share of the discs' single-disc steps one after another (discs
 * dealt largest first to the least-loaded branch), then join */
static int enqueue_disc_graph(mhd_batch *b, int parity)
{
    const int n = b->n, K = b->nbranch;
    while ((int)b->bst.size() < K + 1) {
        cudaStream_t s;
        cudaEvent_t e;
        BCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        b->bst.push_back(s);
        BCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->bev.push_back(e);
    }
    std::vector<int> order(n);
    for (int d = 0; d < n; d++) order[d] = d;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return b->ctx[x]->nc > b->ctx[y]->nc; });
    std::vector<long long> load(K, 0);
    std::vector<std::vector<int>> part(K);
    for (int d : order) {
        int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        part[k].push_back(d);
        load[k] += b->ctx[d]->nc;
    }
    BCK(cudaEventRecord(b->bev[K], b->st));
    long long launches = 0;
    for (int k = 0; k < K; k++) {
        BCK(cudaStreamWaitEvent(b->bst[k], b->bev[K], 0));
        for (int d : part[k]) {
            b->ctx[d]->vcur = parity;
            int rc = mhd_ctx_enqueue_step(b->ctx[d], b->bst[k], &launches);
            if (rc) return rc;
        }
        BCK(cudaEventRecord(b->bev[k], b->bst[k]));
        BCK(cudaStreamWaitEvent(b->st, b->bev[k], 0));
    }
    b->step_launches = launches;
    return MHD_OK;
}

static int enqueue_batch_step(mhd_batch *b, int parity)
{
    const int n = b->n;
    if (b->discgraph) return enqueue_disc_graph(b, parity);
    BCK(cudaMemsetAsync(b->dcnt, 0, 9 * n * sizeof(int), b->st));
    batch_setdt_kernel<<<b->ndt_tiles, 256, 0, b->st>>>(b->dd, parity ? b->ddt + b->ndt_tiles : b->ddt,
                                                         b->rows_per_tile);
    BCK(cudaGetLastError());
    batch_scalars_kernel<<<n, 256, 0, b->st>>>(b->dd);
    BCK(cudaGetLastError());
    batch_trig_kernel<<<dim3(64, n), 128, 0, b->st>>>(b->dd);
    BCK(cudaGetLastError());
    b->launches += 3;
    static const int rk3[3][2] = {{0, 0}, {1, 0}, {2, 1}};
    static const int rk2[2][2] = {{0, 0}, {3, 1}};
    int par = parity;
    for (int s = 0; s < b->nst; s++) {
        int kind = b->nst == 2 ? rk2[s][0] : rk3[s][0], last = b->nst == 2 ? rk2[s][1] : rk3[s][1];
        if (b->phased) {
            batch_flux_kernel<0><<<b->nph[0], 128, 0, b->st>>>(b->dd, b->dph[0], par);
            batch_flux_kernel<1><<<b->nph[1], 128, 0, b->st>>>(b->dd, b->dph[1], par);
            batch_flux_kernel<2><<<b->nph[2], 128, 0, b->st>>>(b->dd, b->dph[2], par);
            batch_update_kernel<<<b->nph[3], 128, 0, b->st>>>(b->dd, b->dph[3], kind, last, par, s);
            batch_ghost_kernel<<<b->nghost_tiles, 128, 0, b->st>>>(b->dd, b->dghost, kind, last, par, s);
            BCK(cudaGetLastError());
            b->launches += 5;
        } else {
            int *q = b->dqueue + (size_t)s * b->qlen;
            BCK(cudaMemsetAsync(q, 0, b->qlen * sizeof(int), b->st));
            BCK(launch_stage(b, q, kind, last, par, s));
            b->launches++;
        }
        par ^= 1;
    }
    batch_advance_kernel<<<ceil_div(n, 128), 128, 0, b->st>>>(b->dd, n);
    BCK(cudaGetLastError());
    b->launches++;
    return MHD_OK;
}

static int build_graphs(mhd_batch *b)
{
    for (int q = 0; q < 2; q++) {
        if (b->gx[q]) cudaGraphExecDestroy(b->gx[q]);
        b->gx[q] = NULL;
    }
    long long l0 = b->launches;
    for (int par = 0; par < 2; par++) {
        cudaGraph_t g;
        BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_batch_step(b, par);
        cudaError_t e = cudaStreamEndCapture(b->st, &g);
        if (rc) return rc;
        BCK(e);
        BCK(cudaGraphInstantiate(&b->gx[par], g, 0));
        cudaGraphDestroy(g);
    }
    b->launches = l0;
    b->graph_ready = 1;
    return MHD_OK;
}

static int setup_persistent(mhd_batch *b)
{
    const int n = b->n;
    b->hd.assign(n, DiscDev());
    int maxrows = 0;
    for (int d = 0; d < n; d++) {
        mhd_ctx *c = b->ctx[d];
        DiscDev &D = b->hd[d];
        memset((void *)&D, 0, sizeof D);
        D.G = c->G;
        D.U = (float *)c->U; D.U1 = (float *)c->U1; D.Va = (float *)c->Va; D.Vb = (float *)c->Vb;
        D.Uinit = (float *)c->Uinit; D.Vinit = (float *)c->Vinit; D.rhofloor = (float *)c->rhofloor;
        D.F = (float *)c->F; D.Gf = (float *)c->Gf; D.H = (float *)c->H; D.Uraw = (float *)c->Uraw;
        D.sc = c->d_sc; D.trig = c->d_trig; D.trigf = c->d_trigf; D.part = c->d_part;
        for (int dir = 0; dir < 3; dir++) {
            Box &bx = D.fbox[dir];
            bx.i0 = dir == 0 ? 0 : 1; bx.i1 = c->ixmax - 1;
            bx.j0 = dir == 1 ? 0 : 1; bx.j1 = c->jymax - 1;
            bx.k0 = dir == 2 ? 0 : 1; bx.k1 = c->kzmax - 1;
        }
        D.ubox.i0 = 1; D.ubox.i1 = c->ixmax - 1; D.ubox.j0 = 1; D.ubox.j1 = c->jymax - 1;
        D.ubox.k0 = 1; D.ubox.k1 = c->kzmax - 1;
        D.cfl = c->p.cfl; D.minminlength = c->G.minminlength; D.dtmin = c->p.dtmin;
        D.psifac = c->p.scheme == MHD_SCHEME_RK2 ? 0.5 : MHD_ONEO3;
        D.tausp = c->p.tausp; D.epssp0 = c->p.epssp0; D.omdiff = c->omdiff; D.armnum = (double)c->p.armnum;
        D.gravity = c->p.gravity;
        int rows = (c->ixmax - 12) * (c->jymax - 2);
        if (rows > maxrows) maxrows = rows;
    }
    /* CFL row tiles: at most the context's partial buffer per disc */
    b->rows_per_tile = 8;
    std::vector<uint2> dt;
    for (int d = 0; d < n; d++) {
        mhd_ctx *c = b->ctx[d];
        int rows = (c->ixmax - 12) * (c->jymax - 2);
        int rpt = b->rows_per_tile;
        while (ceil_div(rows, rpt) > c->npart) rpt *= 2;
        if (rpt > b->rows_per_tile) b->rows_per_tile = rpt;
    }
    for (int d = 0; d < n; d++) {
        mhd_ctx *c = b->ctx[d];
        int rows = (c->ixmax - 12) * (c->jymax - 2);
        b->hd[d].ndt = ceil_div(rows, b->rows_per_tile);
    }
    for (int par = 0; par < 2; par++)
        for (int d = 0; d < n; d++)
            for (int l = 0; l < b->hd[d].ndt; l++)
                dt.push_back(make_uint2(d, ((unsigned)par << 31) | (unsigned)l));
    b->ndt_tiles = (int)dt.size() / 2;
    BCK(cudaMalloc((void **)&b->ddt, dt.size() * sizeof(uint2)));
    BCK(cudaMemcpy(b->ddt, dt.data(), dt.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    BCK(cudaMalloc((void **)&b->dd, n * sizeof(DiscDev)));
    BCK(cudaMalloc((void **)&b->derr, sizeof(int)));
    BCK(cudaMemset(b->derr, 0, sizeof(int)));
    BCK(cudaMalloc((void **)&b->dcnt, 9 * n * sizeof(int)));
    for (int d = 0; d < n; d++) b->hd[d].counters = b->dcnt + 9 * d;
    BCK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    int rc = build_tiles(b, CANDIDATES[0]);
    if (rc) return rc;
    b->nblk_stage = stage_blocks(b->cfg);
    /* phased-mode tiles of 128 cells: by rows x bx cells along k */
    for (int ph = 0; ph < 4; ph++) {
        std::vector<uint4> tl;
        for (int d = 0; d < n; d++) {
            const Box &bx = ph < 3 ? b->hd[d].fbox[ph] : b->hd[d].ubox;
            int nk = bx.k1 - bx.k0;
            int wx = 32 * ceil_div(nk < 128 ? nk : 128, 32);
            int by = 128 / wx;
            for (int i = bx.i0; i < bx.i1; i++)
                for (int j = bx.j0; j < bx.j1; j += by)
                    for (int k0 = bx.k0; k0 < bx.k1; k0 += wx)
                        tl.push_back(make_uint4(d, i, j, ((unsigned)wx << 20) | (unsigned)k0));
        }
        b->nph[ph] = (int)tl.size();
        BCK(cudaMalloc((void **)&b->dph[ph], tl.size() * sizeof(uint4)));
        BCK(cudaMemcpy(b->dph[ph], tl.data(), tl.size() * sizeof(uint4), cudaMemcpyHostToDevice));
    }
    std::vector<uint2> gt;
    for (int d = 0; d < n; d++) {
        const Geom &G = b->hd[d].G;
        long long ng = 2LL * G.ixmax * G.jymax + 2LL * G.ixmax * (G.kzmax - 2) + 2LL * (G.jymax - 2) * (G.kzmax - 2);
        for (long long l = 0; l * 128 < ng; l++) gt.push_back(make_uint2(d, (unsigned)l));
    }
    b->nghost_tiles = (int)gt.size();
    BCK(cudaMalloc((void **)&b->dghost, gt.size() * sizeof(uint2)));
    BCK(cudaMemcpy(b->dghost, gt.data(), gt.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    return MHD_OK;
}

extern "C" int mhd_batch_create(int n, const mhd_grid *grids, const mhd_params *params, mhd_batch **out)
{
    if (!out || n < 1 || !grids || !params) return MHD_ERR_ARG;
    *out = NULL;
    mhd_batch *b = new (std::nothrow) mhd_batch();
    if (!b) return MHD_ERR_NOMEM;
    b->n = n;
    b->spin_limit = MHD_SPIN_LIMIT;
    b->stall_disc = -1;
    b->ctx.assign(n, NULL);
    b->stopped.assign(n, 0);
    int fp32 = params[0].precision == MHD_PREC_FP32;
    b->nst = params[0].scheme == MHD_SCHEME_RK2 ? 2 : 3;
    for (int i = 0; i < n; i++) {
        if ((params[i].precision == MHD_PREC_FP32) != fp32 || params[i].precision == MHD_PREC_FP32X2 ||
            params[i].scheme != params[0].scheme) {
            mhd_batch_destroy(b);
            return MHD_ERR_ARG;   /* one precision and one RK scheme per batch */
        }
        int rc = mhd_create(&grids[i], &params[i], &b->ctx[i]);
        if (rc) {
            mhd_batch_destroy(b);
            return rc;
        }
    }
    b->persistent = fp32;
    if (fp32) {
        for (int i = 0; i < n; i++) {
            int rc = mhd_ctx_prepare_run(b->ctx[i]);
            if (rc) {
                mhd_batch_destroy(b);
                return rc;
            }
        }
        int rc = setup_persistent(b);
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
    if (b->st) cudaStreamSynchronize(b->st);
    for (int q = 0; q < 2; q++)
        if (b->gx[q]) cudaGraphExecDestroy(b->gx[q]);
    void *p[] = {b->dd, b->dtiles, b->ddt, b->dqueue, b->derr, b->dcnt, b->dph[0], b->dph[1], b->dph[2],
                 b->dph[3], b->dghost};
    for (size_t q = 0; q < sizeof p / sizeof p[0]; q++)
        if (p[q]) cudaFree(p[q]);
    for (cudaStream_t s2 : b->bst) { cudaStreamSynchronize(s2); cudaStreamDestroy(s2); }
    for (cudaEvent_t e : b->bev) cudaEventDestroy(e);
    if (b->st) cudaStreamDestroy(b->st);
    for (mhd_ctx *c : b->ctx)
        if (c) mhd_destroy(c);
    delete b;
}

extern "C" int mhd_batch_upload(mhd_batch *b, int disc, const double *U, const double *V, const double *Uinit,
                                const double *Vinit, const double *rhofloor)
{
    if (!b || disc < 0 || disc >= b->n) return MHD_ERR_ARG;
    if (b->st) BCK(cudaStreamSynchronize(b->st));
    b->stopped[disc] = 0;
    int rc = mhd_upload(b->ctx[disc], U, V, Uinit, Vinit, rhofloor);
    if (rc) return rc;
    /* all discs share the batch's primitive parity */
    if (b->persistent && b->parity) {
        mhd_ctx *c = b->ctx[disc];
        BCK(cudaMemcpy(c->Vb, c->Va, 9 * c->nc * sizeof(float), cudaMemcpyDeviceToDevice));
        c->vcur = 1;
    }
    return MHD_OK;
}

extern "C" int mhd_batch_download(mhd_batch *b, int disc, double *U, double *V)
{
    if (!b || disc < 0 || disc >= b->n) return MHD_ERR_ARG;
    if (b->st) BCK(cudaStreamSynchronize(b->st));
    return mhd_download(b->ctx[disc], U, V);
}

static int batch_run(mhd_batch *b, int nsteps, double *t, int *status)
{
    const int n = b->n;
    for (int d = 0; d < n; d++) {
        StepScalars *h = b->ctx[d]->h_sc;
        h->t = t[d];
        h->dtbad = b->stopped[d];
        BCK(cudaMemcpyAsync(b->ctx[d]->d_sc, h, sizeof(StepScalars), cudaMemcpyHostToDevice, b->st));
    }
    BCK(cudaMemsetAsync(b->derr, 0, sizeof(int), b->st));
    if (!b->graph_ready) {
        int rc = build_graphs(b);
        if (rc) return rc;
    }
    long long per_step = b->discgraph ? b->step_launches : 3 + b->nst * (b->phased ? 5 : 1) + 1;
    for (int s = 0; s < nsteps; s++) {
        BCK(cudaGraphLaunch(b->gx[b->parity], b->st));
        b->parity ^= (b->nst & 1);
        b->launches += per_step;
    }
    for (int d = 0; d < n; d++)
        BCK(cudaMemcpyAsync(b->ctx[d]->h_sc, b->ctx[d]->d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, b->st));
    int herr = 0;
    BCK(cudaMemcpyAsync(&herr, b->derr, sizeof(int), cudaMemcpyDeviceToHost, b->st));
    BCK(cudaStreamSynchronize(b->st));
    for (int d = 0; d < n; d++) {
        t[d] = b->ctx[d]->h_sc->t;
        b->ctx[d]->vcur = b->parity;
        if (b->ctx[d]->h_sc->dtbad) b->stopped[d] = 1;
        if (b->ctx[d]->h_sc->err) {   /* a disc's staged update tile gave up waiting (disc-graph mode) */
            herr = 1;
            b->ctx[d]->h_sc->err = 0;
        }
    }
    if (status)
        for (int d = 0; d < n; d++) status[d] = b->stopped[d] ? MHD_ERR_DT : MHD_OK;
    return herr ? MHD_ERR_TIMEOUT : MHD_OK;
}

extern "C" int mhd_batch_step(mhd_batch *b, int nsteps, double *t, int *status)
{
    if (!b || !t || nsteps < 0) return MHD_ERR_ARG;
    if (b->persistent) return batch_run(b, nsteps, t, status);
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

extern "C" int mhd_batch_set_mode(mhd_batch *b, int mode, int arg)
{
    if (!b) return MHD_ERR_ARG;
    if (!b->persistent) return mode == 0 ? MHD_OK : MHD_ERR_ARG;   /* plain form: per-disc mhd_step */
    if (mode == 0) {
        if (arg < 0 || arg >= NCAND) return MHD_ERR_ARG;
        int rc = build_tiles(b, CANDIDATES[arg]);
        if (rc) return rc;
        b->nblk_stage = stage_blocks(b->cfg);
    } else if (mode == 2) {
        if (arg < 1 || arg > 64) return MHD_ERR_ARG;
        b->nbranch = std::min(arg, b->n);
    } else if (mode != 1) {
        return MHD_ERR_ARG;
    }
    if (b->st) BCK(cudaStreamSynchronize(b->st));
    b->phased = mode == 1;
    b->discgraph = mode == 2;
    b->graph_ready = 0;
    return MHD_OK;
}

extern "C" int mhd_batch_debug_stall(mhd_batch *b, int disc, int spin_limit)
{
    if (!b || !b->persistent || disc < -1 || disc >= b->n || (disc >= 0 && spin_limit < 1)) return MHD_ERR_ARG;
    if (b->st) BCK(cudaStreamSynchronize(b->st));
    b->stall_disc = disc;
    b->spin_limit = disc >= 0 ? spin_limit : MHD_SPIN_LIMIT;
    b->phased = 0;
    b->discgraph = 0;
    int rc = build_tiles(b, b->cfg);
    if (rc) return rc;
    b->nblk_stage = stage_blocks(b->cfg);
    b->graph_ready = 0;
    return MHD_OK;
}

extern "C" int mhd_batch_tune(mhd_batch *b, int *best)
{
    if (!b || !best) return MHD_ERR_ARG;
    if (!b->persistent) {
        best[0] = 1; best[1] = 1; best[2] = 128; best[3] = 128; best[4] = 1;
        return MHD_OK;
    }
    const int n = b->n;
    BCK(cudaStreamSynchronize(b->st));
    /* snapshot the evolving state */
    std::vector<std::vector<double>> U(n), V(n);
    std::vector<double> t0(n), tt(n);
    std::vector<int> stop0 = b->stopped;
    int par0 = b->parity;
    for (int d = 0; d < n; d++) {
        mhd_ctx *c = b->ctx[d];
        U[d].resize(9 * c->nc);
        V[d].resize(9 * c->nc);
        int rc = mhd_download(c, U[d].data(), V[d].data());
        if (rc) return rc;
        t0[d] = c->h_sc->t;
    }
    auto restore = [&]() -> int {
        b->parity = 0;
        for (int d = 0; d < n; d++) {
            int rc = mhd_upload_state(b->ctx[d], U[d].data(), V[d].data());
            if (rc) return rc;
            b->ctx[d]->vcur = 0;
        }
        b->stopped = stop0;
        return MHD_OK;
    };
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    int best_i = 0;
    /* candidates: the persistent tile shapes, then the phased mode, then the
     * disc graph on 2, 4, 8 or 16 branches */
    static const int BRANCHES[] = {2, 4, 8, 16};
    const int nall = NCAND + 1 + 4;
    auto select = [&](int ci) -> int {
        b->phased = ci == NCAND;
        b->discgraph = ci > NCAND;
        if (b->discgraph) b->nbranch = std::min(BRANCHES[ci - NCAND - 1], n);
        if (ci < NCAND) {
            int rc = build_tiles(b, CANDIDATES[ci]);
            if (rc) return rc;
            b->nblk_stage = stage_blocks(b->cfg);
        }
        return MHD_OK;
    };
    for (int ci = 0; ci < nall; ci++) {
        int rc = restore();
        if (rc) return rc;
        if ((rc = select(ci))) return rc;
        b->graph_ready = 0;
        tt = t0;
        if ((rc = batch_run(b, 1, tt.data(), NULL))) return rc;   /* warm-up + graph build */
        BCK(cudaEventRecord(e0, b->st));
        if ((rc = batch_run(b, 3, tt.data(), NULL))) return rc;
        BCK(cudaEventRecord(e1, b->st));
        BCK(cudaEventSynchronize(e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) { best_ms = ms; best_i = ci; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int rc = restore();
    if (rc) return rc;
    for (int d = 0; d < n; d++) b->ctx[d]->h_sc->t = t0[d];
    if ((rc = select(best_i))) return rc;
    b->graph_ready = 0;
    (void)par0;
    if (b->discgraph) {
        best[0] = b->nbranch; best[1] = 0; best[2] = 0; best[3] = 0; best[4] = 2;
    } else if (b->phased) {
        best[0] = 1; best[1] = 1; best[2] = 128; best[3] = 128; best[4] = 1;
    } else {
        best[0] = CANDIDATES[best_i].sl;
        best[1] = CANDIDATES[best_i].lag;
        best[2] = 65536 / (128 * CANDIDATES[best_i].minb);
        best[3] = 128;
        best[4] = 0;
    }
    return MHD_OK;
}
