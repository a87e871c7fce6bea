/*
 * mhd_pair.cuh -- the precision form with pair state (MHD_PREC_FP32X2).
 *
 * The conserved state -- U^n, the stage state U^(k) and the raw updated state
 * the boundary fills copy -- is held as two FP32 words per value, hi + lo
 * (|lo| <= ulp(hi)/2, about 48 significant bits), so the state no longer
 * rounds to FP32 after every stage.  Everything per face stays as in the FP32
 * form: the primitives V are FP32, and reconstruction, Riemann fluxes, flux
 * divergence and sources run on the FP32 pipe (the same flux kernels).  The
 * pairs enter only the update and the boundary fills:
 *   - the stage combination (firststep.h:97-118, secondstep.h:100-121,
 *     thirdstep.h:100-123) adds the FP32 correction c (d + w inc) to the
 *     pair base state with an error-free sum;
 *   - the GLM factor (glmsourcesolver.h:19-47) multiplies psi as a pair;
 *   - UtoV (utov.h:24-68) forms the kinetic and magnetic energy from the
 *     pairs error-free on the FP32 pipe and cancels E - (KE + ME) with a
 *     two-sum, so the pressure sees the full state;
 *   - the absorbing layers (xboundary.h:133-138, centralboundary.h:36-41,
 *     zboundary.h:40-46) act in FP64 on the few cells they touch;
 *   - Check's floors (check.h:42-172) reset the words they overwrite.
 * The FP32 pipe carries all of it (FP64 only in the absorbing cells of the
 * last stage).  Only the split stage shape with thread loads runs this
 * form.
 */
#ifndef MHD_PAIR_CUH
#define MHD_PAIR_CUH

#include "mhd_kernels.cuh"

namespace mhd {

/* 1/3 = ONEO3_HI + ONEO3_LO to about 2^-50 */
#define MHD_ONEO3_HI 0.3333333432674407958984375f
#define MHD_ONEO3_LO (-9.934107758624577e-09f)

/* s + e = a + b exactly (Knuth's two-sum; explicitly rounded operations so
 * no contraction undoes it) */
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

/* s + e = a + b exactly when |a| >= |b| (or a == 0) */
__device__ __forceinline__ void fast_two_sum_f(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

/* (ph, pl) = (ah + al)(bh + bl) to about 2^-46, normalised */
__device__ __forceinline__ void pair_mul(float ah, float al, float bh, float bl, float &ph, float &pl)
{
    const float p = __fmul_rn(ah, bh);
    const float e = fmaf(ah, bh, -p) + (ah * bl + al * bh);
    fast_two_sum_f(p, e, ph, pl);
}

/* (hi, lo) += (a + al)^2, with the square's rounding and 2 a al in the low word */
__device__ __forceinline__ void acc_sq_pair(float a, float al, float &hi, float &lo)
{
    acc_sq(a, hi, lo);
    lo = fmaf(2.0f * a, al, lo);
}

/* UtoV (utov.h:38-58) of the pair state (uh + ul) into FP32 primitives w[],
 * on the FP32 pipe alone.  The kinetic and magnetic energies are (hi, lo)
 * pairs formed error-free from both words (m_phi / r with 1/r as a pair),
 * 1/rho is refined by a Newton step from both words of rho, and the
 * cancellation E - (KE + ME) is a two-sum of the high words (exact wherever
 * the two are within a factor of two, which is where it cancels) plus the low
 * words; (gamma-1) = 2/3 is applied as an FP32 pair. */
__device__ __forceinline__ void utov_pair(const Geom &G, int i, const float *uh, const float *ul, float *w)
{
    const float oxh = G.f.oneox[i], oxl = G.oneoxlo[i];
    const float ir = 1.0f / uh[0];
    const float irl = (fmaf(-uh[0], ir, 1.0f) - ul[0] * ir) * ir;      /* 1/rho = ir + irl */
    const float mh = __fmul_rn(uh[2], oxh);                              /* m_phi / r = mh + ml */
    const float ml = fmaf(uh[2], oxh, -mh) + (uh[2] * oxl + ul[2] * oxh);
    float sh, sl;                                                        /* r2v2 = sh + sl */
    two_sq(uh[1], sh, sl);
    sl = fmaf(2.0f * uh[1], ul[1], sl);
    acc_sq_pair(mh, ml, sh, sl);
    acc_sq_pair(uh[3], ul[3], sh, sl);
    float kh = __fmul_rn(sh, ir);                                        /* 2 KE = (sh + sl)(ir + irl) */
    float kl = fmaf(sh, ir, -kh) + (sh * irl + sl * ir);
    acc_sq_pair(uh[4], ul[4], kh, kl);                                   /* + B^2 */
    acc_sq_pair(uh[5], ul[5], kh, kl);
    acc_sq_pair(uh[6], ul[6], kh, kl);
    const float hh = 0.5f * kh, hl = 0.5f * kl;
    w[0] = uh[0];
    w[1] = uh[1] * ir;
    w[2] = uh[2] * ir * G.f.oneox[i];
    w[3] = uh[3] * ir;
    w[4] = uh[4]; w[5] = uh[5]; w[6] = uh[6];
    float ds, de;
    two_sum_f(uh[7], -hh, ds, de);
    const float d = __fadd_rn(ds, __fsub_rn(__fadd_rn(de, ul[7]), hl));
    w[7] = fmaf(d, MHD_GM1_HI, __fmul_rn(d, MHD_GM1_LO));
    w[8] = uh[8];
}

/* UtoV then Check on a pair state: a floor overwrites the high words of the
 * variables it resets (rho and r rho v_phi for the density and beta floors;
 * m_r, m_z and E for all three) and clears their low words */
__device__ __forceinline__ int utov_check_pair(const Geom &G, int i, float rhofloor, float *uh, float *ul, float *w)
{
    utov_pair(G, i, uh, ul, w);
    const int flags = check_floors<float>(G, i, rhofloor, uh, w);
    if (flags) {
        ul[1] = 0.0f; ul[3] = 0.0f; ul[7] = 0.0f;
        if (flags & 5) { ul[0] = 0.0f; ul[2] = 0.0f; }
    }
    return flags;
}

/* the absorbing layers (absorb<T>) on a pair state, in FP64 with the FP64
 * factors; only cells inside a layer pay for it */
__device__ __forceinline__ void absorb_pair(const Geom &G, const float *__restrict__ Uinit, int i, int j, int k,
                                            bool zright, float uh[9], float ul[9])
{
    const Tabs<double> &tb = G.d;
    const long long q = cidx(G, i, j, k);
    const int ix0 = G.ixmax - 11, kz0 = G.kzmax - 11;
    const bool ax = i >= ix0, ac = i <= G.irin, az = zright && k >= kz0;
    if (!(ax || ac || az)) return;
    const double fx = ax ? tb.xabs[i - ix0] : 0.0, fc = ac ? tb.cabs[(long long)i * G.kzmax + k] : 0.0;
    const double fz = az ? tb.zabs[k - kz0] : 0.0;
#pragma unroll
    for (int m = 0; m < 9; m++) {
        const double ui = Uinit[m * G.nc + q];
        double v = (double)uh[m] + (double)ul[m];
        if (ax) v -= (fx * (v - ui));
        if (ac) v -= (fc * (v - ui));
        if (az) v -= (fz * (v - ui));
        uh[m] = (float)v;
        ul[m] = (float)(v - (double)uh[m]);
    }
}

/* the stored pair state and primitives of one cell */
__device__ __forceinline__ void store_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p, long long q,
                                           const float uh[9], const float ul[9], const float W[9])
{
    const long long nc = G.nc;
    const bool to_u1 = a.kind == 0 || a.kind == 1;
    float *Uo = to_u1 ? a.U1 : a.Un, *Ul = to_u1 ? p.U1lo : p.Unlo;
#pragma unroll
    for (int m = 0; m < 9; m++) {
        Uo[m * nc + q] = uh[m];
        Ul[m * nc + q] = ul[m];
        a.Vout[m * nc + q] = W[m];
    }
}

/* zghost_fill on a pair state: the k-plane ghost an interior cell is the
 * source of, from the cell's raw updated pair state */
__device__ __forceinline__ void zghost_fill_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p, int i,
                                                 int j, int k, const float uh[9], const float ul[9])
{
    int kg;
    bool flip = false;
    if (G.scheme == MHD_SCHEME_RK2) {
        if (k == 2) { kg = 0; flip = true; }
        else if (k == G.kzmax - 2) kg = G.kzmax - 1;
        else return;
    } else {
        if (k == G.kzmax - 2) kg = 0;
        else if (k == 1) kg = G.kzmax - 1;
        else return;
    }
    const long long qg = cidx(G, i, j, kg);
    float gh[9], gl[9], W[9];
#pragma unroll
    for (int m = 0; m < 9; m++) {
        const bool neg = flip && m == 3;
        gh[m] = neg ? -uh[m] : uh[m];
        gl[m] = neg ? -ul[m] : ul[m];
    }
    if (a.last) absorb_pair(G, a.Uinit, i, j, kg, G.scheme == MHD_SCHEME_RK2, gh, gl);
    const int flags = utov_check_pair(G, i, a.rhofloor[qg], gh, gl, W);
    store_pair(G, a, p, qg, gh, gl, W);
    if (flags & 1) atomicAdd(&a.counters[0], 1);
    if (flags & 2) atomicAdd(&a.counters[1], 1);
    if (flags & 4) atomicAdd(&a.counters[2], 1);
}

/* The update of one interior cell on the pair state.  The flux divergence,
 * the sources and the increment inc = dt (S - div) are the FP32 form's; the
 * stage combination v = base + c (sgn (u1 - un) + w inc) (StageCoef) forms
 * the correction in FP32 -- it is small against U, and the difference of the
 * high words is exact wherever the two states are within a factor of two --
 * and adds it to the pair base with an error-free sum, c = 1/3 as a pair. */
__device__ __forceinline__ int update_cell_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p, int i,
                                                int j, int k)
{
    const long long nc = G.nc, q = cidx(G, i, j, k);
    const long long si = (long long)G.jymax * G.kzmax, sj = G.kzmax;
    const StepScalars *sc = a.sc;
    const float dt = sc->dtf;
    const int kind = a.kind;
    const StageCoef kc = stage_coef(kind);
    const float ch = kind == 2 ? MHD_ONEO3_HI : kc.c, cl = kind == 2 ? MHD_ONEO3_LO : 0.0f;
    float g[6], div[9], W[9], S[9], uh[9], ul[9];
    /* in three phases, as the FP32 update: the flux divergence (54 loads;
     * the last z face of a row from the compact Hb), the primitives and
     * sources, then the pair states and the combination */
    const float *hu = a.H + q;
    long long hs = nc;
    if (a.Hb && k == G.kzmax - 2) {
        hu = a.Hb + (long long)(i - 1) * (G.jymax - 2) + (j - 1);
        hs = (long long)(G.ixmax - 2) * (G.jymax - 2);
    }
    geo_factors<float>(G, i, k, g);
#pragma unroll
    for (int m = 0; m < 9; m++) {
        const long long mq = m * nc + q;
        div[m] = flux_div<float>(g, a.F[mq], a.F[mq - si], a.G[mq], a.G[mq - sj], hu[m * hs], a.H[mq - 1]);
    }
#pragma unroll
    for (int m = 0; m < 9; m++) W[m] = a.V[m * nc + q];
    source_at<float>(G, *sc, a.trig, a.trigf, i, j, k, W, S);
#pragma unroll
    for (int m = 0; m < 9; m++) {
        const long long mq = m * nc + q;
        float unh = a.Un[mq], unl = p.Unlo[mq];
        float u1h = 0.0f, u1l = 0.0f;
        if (kind != 0) { u1h = a.U1[mq]; u1l = p.U1lo[mq]; }
        if (m == 8) {   /* GLMSourceSolver on U and U1, the factor as a pair */
            pair_mul(sc->psif, sc->psifl, unh, unl, unh, unl);
            pair_mul(sc->psif, sc->psifl, u1h, u1l, u1h, u1l);
        }
        const float inc = dt * (S[m] - div[m]);
        const float t = kc.sgn * (__fsub_rn(u1h, unh) + __fsub_rn(u1l, unl)) + kc.w * inc;
        const float corr = fmaf(ch, t, cl * t);
        const float bh = kc.from_u1 ? u1h : unh, bl = kc.from_u1 ? u1l : unl;
        float s, e;
        two_sum_f(bh, corr, s, e);
        fast_two_sum_f(s, __fadd_rn(e, bl), uh[m], ul[m]);
    }
    if (is_bc_source(G, i, j, k)) {
#pragma unroll
        for (int m = 0; m < 9; m++) { a.Uraw[m * nc + q] = uh[m]; p.Urawlo[m * nc + q] = ul[m]; }
        if (a.zghost) zghost_fill_pair(G, a, p, i, j, k, uh, ul);
    }
    if (G.scheme == MHD_SCHEME_RK2 && k == 1) { uh[3] = 0.0f; ul[3] = 0.0f; }   /* zboundary.h:87 */
    if (a.last) absorb_pair(G, a.Uinit, i, j, k, G.scheme == MHD_SCHEME_RK2, uh, ul);
    const int flags = utov_check_pair(G, i, a.rhofloor[q], uh, ul, W);
    store_pair(G, a, p, q, uh, ul, W);
    return flags;
}

__global__ void __launch_bounds__(128, 8) update_pair_kernel(Geom G, StageArgs<float> a, PairArgs p)
{
    if (a.sc->dtbad) return;
    const int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = 1 + blockIdx.z;
    int flags = 0;
    if (k < G.kzmax - 1 && j < G.jymax - 1) flags = update_cell_pair(G, a, p, i, j, k);
    add_counters(flags, a.counters);
}

/* ghost_cell on the pair state: the composed boundary fills copy both words */
__global__ void __launch_bounds__(128) ghost_pair_kernel(Geom G, StageArgs<float> a, PairArgs p)
{
    if (a.sc->dtbad) return;
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    int flags = 0;
    if (tid < ghost_count(G, a.zghost)) {
        int i, j, k, si, sj, sk;
        unsigned neg;
        ghost_cell_of(G, tid, a.zghost, i, j, k);
        ghost_source(G, i, j, k, si, sj, sk, neg);
        const long long nc = G.nc, q = cidx(G, i, j, k), qs = cidx(G, si, sj, sk);
        float uh[9], ul[9], W[9];
#pragma unroll
        for (int m = 0; m < 9; m++) {
            const float h = a.Uraw[m * nc + qs], l = p.Urawlo[m * nc + qs];
            const bool n = (neg >> m) & 1u;
            uh[m] = n ? -h : h;
            ul[m] = n ? -l : l;
        }
        if (G.scheme == MHD_SCHEME_RK2 && k == 1) { uh[3] = 0.0f; ul[3] = 0.0f; }
        if (a.last) absorb_pair(G, a.Uinit, i, j, k, G.scheme == MHD_SCHEME_RK2, uh, ul);
        flags = utov_check_pair(G, i, a.rhofloor[q], uh, ul, W);
        store_pair(G, a, p, q, uh, ul, W);
    }
    add_counters(flags, a.counters);
}

/* FP64 host state -> pair (hi = the nearest FP32 value, lo = the rest) */
__global__ void cvt_pair_from_f64(const double *__restrict__ src, float *__restrict__ hi, float *__restrict__ lo,
                                  long long n)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double v = src[t];
        const float h = (float)v;
        hi[t] = h;
        lo[t] = (float)(v - (double)h);
    }
}

__global__ void cvt_pair_to_f64(const float *__restrict__ hi, const float *__restrict__ lo, double *__restrict__ dst,
                                long long n)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (double)hi[t] + (double)lo[t];
}

/* V = UtoV(U) of the pair state at every cell, ghosts included (no floors) */
__global__ void __launch_bounds__(256) derive_v_pair_kernel(Geom G, const float *__restrict__ U,
                                                            const float *__restrict__ Ulo, float *__restrict__ V)
{
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < G.nc;
         q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q / ((long long)G.jymax * G.kzmax));
        float uh[9], ul[9], w[9];
#pragma unroll
        for (int m = 0; m < 9; m++) { uh[m] = U[m * G.nc + q]; ul[m] = Ulo[m * G.nc + q]; }
        utov_pair(G, i, uh, ul, w);
#pragma unroll
        for (int m = 0; m < 9; m++) V[m * G.nc + q] = w[m];
    }
}

} /* namespace mhd */

/* the pair-state launchers (declared in mhd_launch.h), expanded once in the
 * FP32 translation unit */
#define MHD_DEFINE_PAIR_LAUNCHERS                                                                            \
    namespace mhd {                                                                                          \
    cudaError_t launch_update_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p,              \
                                   cudaStream_t st)                                                          \
    {                                                                                                        \
        dim3 gr, bl;                                                                                         \
        grid3(G.kzmax - 2, G.jymax - 2, G.ixmax - 2, gr, bl);                                                \
        update_pair_kernel<<<gr, bl, 0, st>>>(G, a, p);                                                      \
        return cudaGetLastError();                                                                           \
    }                                                                                                        \
    cudaError_t launch_ghost_pair(const Geom &G, const StageArgs<float> &a, const PairArgs &p,               \
                                  cudaStream_t st)                                                           \
    {                                                                                                        \
        const long long ng = ghost_count(G, a.zghost);                                                       \
        ghost_pair_kernel<<<nblocks(ng, 128), 128, 0, st>>>(G, a, p);                                        \
        return cudaGetLastError();                                                                           \
    }                                                                                                        \
    cudaError_t launch_cvt_pair(const double *src, float *hi, float *lo, long long n, cudaStream_t st)       \
    {                                                                                                        \
        cvt_pair_from_f64<<<1024, 256, 0, st>>>(src, hi, lo, n);                                             \
        return cudaGetLastError();                                                                           \
    }                                                                                                        \
    cudaError_t launch_cvt_pair_back(const float *hi, const float *lo, double *dst, long long n,             \
                                     cudaStream_t st)                                                        \
    {                                                                                                        \
        cvt_pair_to_f64<<<1024, 256, 0, st>>>(hi, lo, dst, n);                                               \
        return cudaGetLastError();                                                                           \
    }                                                                                                        \
    cudaError_t launch_derive_v_pair(const Geom &G, const float *U, const float *Ulo, float *V,              \
                                     cudaStream_t st)                                                        \
    {                                                                                                        \
        derive_v_pair_kernel<<<(unsigned)(4 * sm_count()), 256, 0, st>>>(G, U, Ulo, V);                      \
        return cudaGetLastError();                                                                           \
    }                                                                                                        \
    }

#endif
