/*
 * mhd_launch.h -- launcher interface between the context code (mhd_ctx.cu)
 * and the per-precision kernel translation units (mhd_fp64.cu, mhd_fp32.cu).
 * Overloaded on the state type: double = plain form, float = precision form.
 */
#ifndef MHD_LAUNCH_H
#define MHD_LAUNCH_H

#include <cuda.h>   /* CUtensorMap (a type only: the library does not link the driver API) */

#include "mhd_dev.cuh"

/* cells per tile of the TMA-staged update, and the width of its windows that
 * start up to 3 cells before the tile (TMA rows start on 16-byte boundaries) */
#define MHD_UPD_TILE 128
#define MHD_UPD_WIDE 136

namespace mhd {

/* half-open index box [i0,i1) x [j0,j1) x [k0,k1) */
struct Box {
    int i0, i1, j0, j1, k0, k1;
};

struct MaxLoc {
    double v;
    long long q;
};

/* Tensor maps of the arrays the TMA-staged update reads (precision form),
 * each array viewed as a 2D FP32 tensor [nvar][nc] with row stride nc */
struct UpdMaps {
    CUtensorMap v[2];          /* Va, Vb: box {MHD_UPD_TILE, 9} */
    CUtensorMap f, g, un, u1;  /* F, G, U, U1: box {MHD_UPD_TILE, 9} */
    CUtensorMap fm, gm, h;     /* F, G, H: box {MHD_UPD_WIDE, 9} */
    CUtensorMap rho;           /* rhofloor: box {MHD_UPD_TILE, 1} */
};

template <typename T>
struct StageArgs {
    const T *V;            /* stage input primitives */
    const T *F, *G, *H;    /* fluxes */
    T *Un, *U1;            /* U^n and U^(1) (or U^(2)); output goes to one of them */
    const T *Uinit, *rhofloor;
    T *Vout, *Uraw;
    const StepScalars *sc;
    const double *trig;
    const float *trigf;
    int kind, last;
    int *counters;
    const T *Vinit;        /* initial primitives (z MC boundary states; fused stage) */
    int zghost = 0;        /* 1: the update fills the k-plane ghosts of interior (i,j) columns */
    int prefetch = 0;      /* update: blocks ahead whose streamed inputs each block prefetches into L2 (0: none) */
    int ibeg = 1, iend = 0;  /* update: the planes i in [ibeg, iend) it covers (iend 0: through ixmax-2) */
    int wfromu = 0;        /* update (precision form): the cell's primitives from UtoV of U^(k), not loaded */
    const T *Hb = nullptr; /* update: the last z face of each row, [9][rows] (split stage), else in H */
};

/* pair-state form (MHD_PREC_FP32X2): the low words of the state arrays; the
 * high words are the FP32 form's arrays in StageArgs<float> */
struct PairArgs {
    float *Unlo, *U1lo;   /* U^n and U^(k); the stage output goes to one of them, as its high words do */
    float *Urawlo;        /* the raw updated state of the cells the boundary fills copy */
};

cudaError_t launch_update_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p, cudaStream_t st);
cudaError_t launch_ghost_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p, cudaStream_t st);
cudaError_t launch_cvt_pair(const double *src, float *hi, float *lo, long long n, cudaStream_t st);
cudaError_t launch_cvt_pair_back(const float *hi, const float *lo, double *dst, long long n, cudaStream_t st);
cudaError_t launch_derive_v_pair(const Geom &G, const float *U, const float *Ulo, float *V, cudaStream_t st);

#define MHD_DECLARE_LAUNCHERS(T)                                                                             \
    cudaError_t launch_flux(int dir, const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F, \
                            Box b, bool reflayout, cudaStream_t st);                                         \
    cudaError_t launch_states(int dir, const Geom &G, const T *V, const T *Vinit, const StepScalars *sc,     \
                              T *Vl, T *Vr, Box b, cudaStream_t st);                                         \
    cudaError_t launch_flux_zinterior(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc,      \
                                      T *F, Box b, cudaStream_t st);                                         \
    cudaError_t launch_zedge(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F, Box b,  \
                             cudaStream_t st);                                                               \
    cudaError_t launch_flux_zwalk(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F,    \
                                  T *Zs, cudaStream_t st); /* split stage: z faces 0 .. kzmax-3 */          \
    cudaError_t launch_flux_zlast(const Geom &G, const T *Vinit, const StepScalars *sc, T *H, T *Hb,        \
                                  const T *Zs, int Hfull, cudaStream_t st); /* ... face kzmax-2 */          \
    cudaError_t launch_update(const Geom &G, const StageArgs<T> &a, cudaStream_t st);                        \
    cudaError_t launch_update_tma(const Geom &G, const StageArgs<T> &a, const UpdMaps &maps, int vpar,      \
                                  int *err, cudaStream_t st); /* precision form only */                    \
    cudaError_t launch_ghost(const Geom &G, const StageArgs<T> &a, cudaStream_t st);                         \
    cudaError_t launch_stage(const Geom &G, const StageArgs<T> &a, int tj, int seg, cudaStream_t st);        \
    cudaError_t prepare_stage(T *); /* shared-memory attribute of the fused kernels */                       \
    cudaError_t launch_zupdate(const Geom &G, const StageArgs<T> &a, cudaStream_t st);                      \
    cudaError_t launch_setdt(const Geom &G, const T *V, MaxLoc *part, int nblk, cudaStream_t st);            \
    cudaError_t launch_source(const Geom &G, const T *V, const StepScalars *sc, const double *trig,          \
                              const float *trigf, double *S, cudaStream_t st);                               \
    cudaError_t launch_cvt(const double *src, T *dst, long long n, cudaStream_t st);                         \
    cudaError_t launch_cvt_back(const T *src, double *dst, long long n, cudaStream_t st);                    \
    cudaError_t launch_derive_v(const Geom &G, const T *U, T *V, cudaStream_t st);

MHD_DECLARE_LAUNCHERS(double)
MHD_DECLARE_LAUNCHERS(float)

} /* namespace mhd */

#endif
