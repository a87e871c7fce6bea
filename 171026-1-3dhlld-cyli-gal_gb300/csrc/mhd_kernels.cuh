/*
 * mhd_kernels.cuh -- the step's kernels, templated on the real type T and
 * instantiated once per precision form by mhd_fp64.cu / mhd_fp32.cu (which
 * differ only in compile flags).
 *
 * One RK stage = flux(r) + flux(phi) + flux(z: boundary faces, interior
 * faces) + update + ghost (the default), or flux(r) + flux(phi) + z fluxes
 * fused into the update + ghost, or the fused stage kernel + ghost:
 *   flux    every face the update reads: reconstruction (each cell once, both
 *           slots, shared along the direction by a marching thread in r and
 *           phi and by warp shuffles in z), Riemann solver, GLM flux ->
 *           F/G/H[9][cells]
 *   update  one thread per interior cell: sources, the stage's conservative
 *           update, and -- because everything after it up to the next stage
 *           is pointwise for interior cells -- the k=1 v_z zeroing (RK2), the
 *           absorbing layers (last stage), UtoV and Check; the raw updated
 *           state of the cells that boundary fills copy from is also kept
 *   ghost   one thread per ghost cell: the reference's boundary-fill sequence
 *           composed into one source cell and sign per ghost, then the same
 *           pointwise tail as the interior.
 */
#ifndef MHD_KERNELS_CUH
#define MHD_KERNELS_CUH

#include "mhd_dev.cuh"
#include "mhd_launch.h"

/* faces per thread of the marched r and phi flux kernels */
#ifndef MHD_MARCH_RUN
#define MHD_MARCH_RUN 16
#endif

namespace mhd {

/* ------------------------------------------------------------------------ */
/* fluxes                                                                    */
/* ------------------------------------------------------------------------ */
/* one face: reconstruction of the two adjacent cells, Riemann + GLM flux */
template <typename T, int DIR, bool REFLAYOUT>
__device__ __forceinline__ void flux_face(const Geom &G, const T *__restrict__ V, const T *__restrict__ Vinit,
                                          const StepScalars *__restrict__ sc, T *__restrict__ F, int i, int j, int k)
{
    T dt = Scal<T>::dt(sc), ch = Scal<T>::ch(sc), psicoef = Scal<T>::psi(sc);
    T L[9], R[9], Fo[9];
    face_states<T, DIR>(G, V, Vinit, i, j, k, dt, psicoef, L, R);
    face_flux<T, DIR>(G, L, R, i, ch, Fo);
    if (REFLAYOUT) {
        /* the reference's face layout [9][ixmax-1][jymax-1][kzmax-1] (probes) */
        long long nf = (long long)(G.ixmax - 1) * (G.jymax - 1) * (G.kzmax - 1);
        long long q = ((long long)i * (G.jymax - 1) + j) * (G.kzmax - 1) + k;
#pragma unroll
        for (int m = 0; m < 9; m++) F[m * nf + q] = Fo[m];
    } else {
        long long q = cidx(G, i, j, k);
#pragma unroll
        for (int m = 0; m < 9; m++) F[m * G.nc + q] = Fo[m];
    }
}

/* one face's flux into F (cell layout) or the reference's face layout */
template <typename T, bool REFLAYOUT>
__device__ __forceinline__ void store_face(const Geom &G, T *__restrict__ F, int i, int j, int k, const T Fo[9])
{
    if (REFLAYOUT) {
        const long long nf = (long long)(G.ixmax - 1) * (G.jymax - 1) * (G.kzmax - 1);
        const long long q = ((long long)i * (G.jymax - 1) + j) * (G.kzmax - 1) + k;
#pragma unroll
        for (int m = 0; m < 9; m++) F[m * nf + q] = Fo[m];
    } else {
        const long long q = cidx(G, i, j, k);
#pragma unroll
        for (int m = 0; m < 9; m++) F[m * G.nc + q] = Fo[m];
    }
}

/* Faces along r (DIR 0) or phi (DIR 1), one thread marching over a run of MR
 * consecutive faces f of one (j,k) or (i,k) line.  Face f takes the left slot
 * of cell f and the right slot of cell f+1 (1 <= f <= N-1, N = nmax-2), so
 * each step reconstructs cell f+1 once, both slots (cell_slots), uses its
 * right slot now and carries its left slot to face f+1: one cell pass per
 * face where a thread per face (flux_face) makes two slot passes.  The first
 * and last face of the direction keep flux_face (their periodic / free /
 * fixed fills); a run starts with the left slot of its first interior cell.  Whole blocks share
 * the run, so the edge faces never diverge inside a warp.  Same operations
 * per state as face_states, so the plain form keeps its bits. */
/* One thread's run of faces [f0, fe) along r (DIR 0) or phi (DIR 1) on the
 * line t (j for r, i for phi) at height k: the body of march_flux_kernel,
 * also the r and phi work items of the batched form's persistent stage. */
template <typename T, int DIR, bool REFLAYOUT>
__device__ __forceinline__ void march_run(const Geom &G, const T *__restrict__ V, const T *__restrict__ Vinit,
                                          const StepScalars *__restrict__ sc, T *__restrict__ F, int t, int k,
                                          int f0, int fe)
{
    const int N = (DIR == 0 ? G.ixmax : G.jymax) - 2;
    const T dt = Scal<T>::dt(sc), ch = Scal<T>::ch(sc), psicoef = Scal<T>::psi(sc);
    if (f0 >= fe) return;
    if (f0 == 0) {
        flux_face<T, DIR, REFLAYOUT>(G, V, Vinit, sc, F, DIR == 0 ? 0 : t, DIR == 0 ? t : 0, k);
        f0 = 1;
    }
    const int fi = min(fe, N);   /* interior faces f0 .. fi-1 */
    if (f0 < fi) {
        T Lc[9];
        slot_of<T, DIR, true>(G, V, f0, DIR == 0 ? f0 : t, DIR == 0 ? t : f0, k, dt, psicoef, Lc);
#pragma unroll 1
        for (int f = f0; f < fi; f++) {
            const int i = DIR == 0 ? f : t, j = DIR == 0 ? t : f;
            T Wl[9], R[9], Fo[9];
            if (DIR == 0) cell_slots<T, 0>(G, V, f + 1, j, k, dt, psicoef, Wl, R);
            else cell_slots<T, 1>(G, V, i, f + 1, k, dt, psicoef, Wl, R);
            face_flux<T, DIR>(G, Lc, R, i, ch, Fo);
            store_face<T, REFLAYOUT>(G, F, i, j, k, Fo);
#pragma unroll
            for (int m = 0; m < 9; m++) Lc[m] = Wl[m];
        }
    }
    if (fe > N) flux_face<T, DIR, REFLAYOUT>(G, V, Vinit, sc, F, DIR == 0 ? N : t, DIR == 0 ? t : N, k);
}

/* Faces along r (DIR 0) or phi (DIR 1), one thread marching over a run of MR
 * consecutive faces f of one (j,k) or (i,k) line.  Face f takes the left slot
 * of cell f and the right slot of cell f+1 (1 <= f <= N-1, N = nmax-2), so
 * each step reconstructs cell f+1 once, both slots (cell_slots), uses its
 * right slot now and carries its left slot to face f+1: one cell pass per
 * face where a thread per face (flux_face) makes two slot passes.  The first
 * and last face of the direction keep flux_face (their periodic / free /
 * fixed fills); a run starts with the left slot of its first interior cell.  Whole blocks share
 * the run, so the edge faces never diverge inside a warp.  Same operations
 * per state as face_states, so the plain form keeps its bits. */
template <typename T, int DIR, int MR, bool REFLAYOUT>
__global__ void __launch_bounds__(128)
march_flux_kernel(Geom G, const T *__restrict__ V, const T *__restrict__ Vinit, const StepScalars *__restrict__ sc,
                  T *__restrict__ F, Box b)
{
    const int k = b.k0 + blockIdx.x * blockDim.x + threadIdx.x;
    const int t = (DIR == 0 ? b.j0 : b.i0) + blockIdx.y * blockDim.y + threadIdx.y;
    const int f0 = (DIR == 0 ? b.i0 : b.j0) + blockIdx.z * MR;
    const int fe = min(f0 + MR, DIR == 0 ? b.i1 : b.j1);
    if (k >= b.k1 || t >= (DIR == 0 ? b.j1 : b.i1)) return;
    march_run<T, DIR, REFLAYOUT>(G, V, Vinit, sc, F, t, k, f0, fe);
}

/* Interior z faces (1 .. kzmax-3 within the box), one warp walking each
 * (i,j) row in chunks of 32 cells: lane l reconstructs cell c = c0 + l once,
 * both slots (cell_slots), and forms face c-1 from its own right slot and the
 * left slot of cell c-1, which the lane below holds (a shuffle; lane 0 takes
 * lane 31's from the previous chunk).  One cell pass per face where the
 * four-cell stencil of interior_states makes two slot passes; loads stay
 * coalesced along k.  Same operations per state as face_states, so the
 * plain form keeps its bits.  FP32: held to 64 registers (8 blocks per SM),
 * 1.48 against 1.56 ms at 78 registers for 512x512x256. */
/* One warp's walk of the interior z faces flo .. fhi-1 of row (i, j): the
 * body of zwalk_flux_kernel, also the z work items of the batched form's
 * persistent stage.  Warp-uniform arguments. */
template <typename T, bool REFLAYOUT>
__device__ __forceinline__ void zwalk_row(const Geom &G, const T *__restrict__ V, const StepScalars *__restrict__ sc,
                                          T *__restrict__ F, int i, int j, int flo, int fhi)
{
    const int lane = threadIdx.x & 31;
    const T dt = Scal<T>::dt(sc), ch = Scal<T>::ch(sc), psicoef = Scal<T>::psi(sc);
    T carry[9];
#pragma unroll
    for (int m = 0; m < 9; m++) carry[m] = T(0.0);
#pragma unroll 1
    for (int c0 = flo; c0 <= fhi; c0 += 32) {   /* warp-uniform */
        const int c = c0 + lane;
        const bool live = c <= fhi;
        T Wl[9], Wr[9], L[9];
        if (live) cell_slots<T, 2>(G, V, i, j, c, dt, psicoef, Wl, Wr);
        else {
#pragma unroll
            for (int m = 0; m < 9; m++) { Wl[m] = T(0.0); Wr[m] = T(0.0); }
        }
#pragma unroll
        for (int m = 0; m < 9; m++) {
            const T up = __shfl_up_sync(0xffffffffu, Wl[m], 1);
            L[m] = lane == 0 ? carry[m] : up;
            carry[m] = __shfl_sync(0xffffffffu, Wl[m], 31);
        }
        if (live && c > flo) {
            T Fo[9];
            face_flux<T, 2>(G, L, Wr, i, ch, Fo);
            store_face<T, REFLAYOUT>(G, F, i, j, c - 1, Fo);
        }
    }
}

/* Interior z faces (1 .. kzmax-3 within the box), one warp walking each
 * (i,j) row in chunks of 32 cells: lane l reconstructs cell c = c0 + l once,
 * both slots (cell_slots), and forms face c-1 from its own right slot and the
 * left slot of cell c-1, which the lane below holds (a shuffle; lane 0 takes
 * lane 31's from the previous chunk).  One cell pass per face where the
 * four-cell stencil of interior_states makes two slot passes; loads stay
 * coalesced along k.  Same operations per state as face_states, so the
 * plain form keeps its bits.  FP32: held to 64 registers (8 blocks per SM),
 * 1.48 against 1.56 ms at 78 registers for 512x512x256. */
template <typename T, bool REFLAYOUT>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 1)
zwalk_flux_kernel(Geom G, const T *__restrict__ V, const StepScalars *__restrict__ sc, T *__restrict__ F, Box b)
{
    const int nj = b.j1 - b.j0;
    const long long nrow = (long long)(b.i1 - b.i0) * nj;
    const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= nrow) return;   /* a whole warp */
    const int i = b.i0 + (int)(row / nj), j = b.j0 + (int)(row % nj);
    const int flo = max(b.k0, 1), fhi = min(b.k1, G.kzmax - 2);   /* faces flo .. fhi-1, cells flo .. fhi */
    zwalk_row<T, REFLAYOUT>(G, V, sc, F, i, j, flo, fhi);
}

/* Every z face of the split stage from one walk per (i,j) row.  The
 * boundary faces' states are slots the walk reconstructs anyway (face_states:
 * minmod ZLeftVlVzAntisymBzsymBoundary takes the right slot of cell 2 with
 * v_z negated and the right slot of cell 1 at face 0, ZRightVrFreeBoundary
 * the left slot of cell kzmax-2 on both sides of face kzmax-2; MC
 * ZVlrFixedBoundary those slots against Vinit at k = 0 and kzmax-1; van Leer
 * ZVlrFreeBoundary the one interior slot on both sides; superbee, periodic,
 * the left slot of cell kzmax-2 and the right slot of cell 1 at both faces).
 *   Face 0 is the face c-1 of the first chunk's lane 0, otherwise idle, so
 * its flux is stored with the chunk's other faces (lane 1's right slot comes
 * by a shuffle); for superbee its left slot is in the last chunk, so the
 * face is left to zlast_flux_kernel.
 *   Face kzmax-2 needs one face evaluation more than whole 32-lane chunks
 * hold: the walk keeps the left slot of cell kzmax-2 (the last chunk's
 * carry) and, for superbee, the right slot of cell 1 in the scratch
 * Zs[18][rows], and zlast_flux_kernel forms that face, one thread per row,
 * into the compact Hb[9][rows] that the update reads for its cells k =
 * kzmax-2 -- a coalesced store where writing H at (i, j, kzmax-2) would touch
 * one 32-byte sector per row and variable.
 * The states are the values face_states forms (cell_slots equals recon_slot
 * bit for bit), so the plain form keeps its bits. */
template <typename T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 1)
zwalk_edges_kernel(Geom G, const T *__restrict__ V, const T *__restrict__ Vinit, const StepScalars *__restrict__ sc,
                   T *__restrict__ F, T *__restrict__ Zs, Box b)
{
    /* b: the interior rows i in [1, ixmax-1), j in [1, jymax-1) (indexing
     * through the box keeps this kernel within 64 registers) */
    const int nj = b.j1 - b.j0;
    const long long nrow = (long long)(b.i1 - b.i0) * nj;
    const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= nrow) return;   /* a whole warp */
    const int i = b.i0 + (int)(row / nj), j = b.j0 + (int)(row % nj);
    const int lane = threadIdx.x & 31;
    const int klast = G.kzmax - 2, lim = G.limiter;
    const T dt = Scal<T>::dt(sc), ch = Scal<T>::ch(sc), psicoef = Scal<T>::psi(sc);
    T carry[9];
#pragma unroll
    for (int m = 0; m < 9; m++) carry[m] = T(0.0);
#pragma unroll 1
    for (int c0 = 1; c0 <= klast; c0 += 32) {   /* warp-uniform */
        const int c = c0 + lane;
        const bool live = c <= klast;
        T Wl[9], Wr[9], L[9];
        if (live) cell_slots<T, 2>(G, V, i, j, c, dt, psicoef, Wl, Wr);
        else {
#pragma unroll
            for (int m = 0; m < 9; m++) { Wl[m] = T(0.0); Wr[m] = T(0.0); }
        }
        /* the next chunk's carry: the left slot of the chunk's last cell --
         * in the last chunk, cell kzmax-2, kept past the walk */
        const int top = min(31, klast - c0);
#pragma unroll
        for (int m = 0; m < 9; m++) {
            const T up = __shfl_up_sync(0xffffffffu, Wl[m], 1);
            L[m] = lane == 0 ? carry[m] : up;
            carry[m] = __shfl_sync(0xffffffffu, Wl[m], top);
        }
        bool face = live && c > 1;
        if (c0 == 1) {   /* face 0 on lane 0 */
            if (lim == MHD_LIMITER_MINMOD) {
#pragma unroll
                for (int m = 0; m < 9; m++) {
                    const T w2 = __shfl_down_sync(0xffffffffu, Wr[m], 1);
                    if (lane == 0) L[m] = m == 3 ? -w2 : w2;
                }
            } else if (lane == 0) {
                const long long q0 = cidx(G, i, j, 0);
#pragma unroll
                for (int m = 0; m < 9; m++)
                    L[m] = lim == MHD_LIMITER_MC ? Vinit[(long long)m * G.nc + q0] : Wr[m];
            }
            if (lane == 0) {
                if (lim == MHD_LIMITER_SUPERBEE) {
#pragma unroll
                    for (int m = 0; m < 9; m++) Zs[(9 + m) * nrow + row] = Wr[m];
                } else {
                    face = live;
                }
            }
        }
        if (face) {
            T Fo[9];
            face_flux<T, 2>(G, L, Wr, i, ch, Fo);
            store_face<T, false>(G, F, i, j, c - 1, Fo);
        }
    }
    if (lane == 0) {   /* the left slot of cell kzmax-2 (the row index recomputed, not held) */
        T *zr = Zs + ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
#pragma unroll
        for (int m = 0; m < 9; m++) zr[m * nrow] = carry[m];
    }
}

/* The last z face (kzmax-2) of each (i,j) row from the slots
 * zwalk_edges_kernel stored in Zs[18][rows] (rows 0..8 the left slot of cell
 * kzmax-2; 9..17, superbee only, the right slot of cell 1), with the fills of
 * face_states: the right state is the left one (minmod ZRightVrFreeBoundary,
 * van Leer ZVlrFreeBoundary), Vinit at kzmax-1 (MC ZVlrFixedBoundary) or the
 * right slot of cell 1 (superbee, periodic, where face 0 takes the same two
 * states and so the same flux).  One thread per row; the flux goes to the
 * compact Hb[9][rows] (coalesced) and, where H must hold every face (Hfull:
 * the TMA-staged update reads H directly) or for superbee's face 0, into H. */
template <typename T>
__global__ void __launch_bounds__(128)
zlast_flux_kernel(Geom G, const T *__restrict__ Vinit, const StepScalars *__restrict__ sc, T *__restrict__ H,
                  T *__restrict__ Hb, const T *__restrict__ Zs, int Hfull)
{
    const int nj = G.jymax - 2;
    const long long nrow = (long long)(G.ixmax - 2) * nj;
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    const int i = 1 + (int)(row / nj), j = 1 + (int)(row % nj);
    const int lim = G.limiter, klast = G.kzmax - 2;
    T L[9], R[9], Fo[9];
#pragma unroll
    for (int m = 0; m < 9; m++) {
        L[m] = Zs[m * nrow + row];
        if (lim == MHD_LIMITER_MC) R[m] = Vinit[(long long)m * G.nc + cidx(G, i, j, klast + 1)];
        else if (lim == MHD_LIMITER_SUPERBEE) R[m] = Zs[(9 + m) * nrow + row];
        else R[m] = L[m];
    }
    face_flux<T, 2>(G, L, R, i, Scal<T>::ch(sc), Fo);
#pragma unroll
    for (int m = 0; m < 9; m++) Hb[m * nrow + row] = Fo[m];
    if (Hfull) store_face<T, false>(G, H, i, j, klast, Fo);
    if (lim == MHD_LIMITER_SUPERBEE) store_face<T, false>(G, H, i, j, 0, Fo);
}

/* The two z boundary faces of each (i,j) column (face 0 and face kzmax-2,
 * which take the special left/right states of face_states), one thread per
 * face with the side slowest so every warp takes one branch; the interior
 * z faces run in zwalk_flux_kernel without that divergence. */
template <typename T, bool REFLAYOUT>
__global__ void __launch_bounds__(128)
flux_zedge_kernel(Geom G, const T *__restrict__ V, const T *__restrict__ Vinit, const StepScalars *__restrict__ sc,
                  T *__restrict__ F, Box b, int lo, int hi)
{
    const int nj = b.j1 - b.j0;
    const long long nij = (long long)(b.i1 - b.i0) * nj;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nij * (lo + hi)) return;
    const int s = (int)(t / nij);
    const long long r = t - s * nij;
    const int k = (lo && s == 0) ? 0 : G.kzmax - 2;
    const int i = b.i0 + (int)(r / nj), j = b.j0 + (int)(r % nj);
    flux_face<T, 2, REFLAYOUT>(G, V, Vinit, sc, F, i, j, k);
}

/* reconstructed face states in the reference's face layout (probe) */
template <typename T, int DIR>
__global__ void __launch_bounds__(128)
states_kernel(Geom G, const T *__restrict__ V, const T *__restrict__ Vinit, const StepScalars *__restrict__ sc,
              T *__restrict__ Vl, T *__restrict__ Vr, Box b)
{
    const int k = b.k0 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = b.j0 + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = b.i0 + blockIdx.z;
    if (k >= b.k1 || j >= b.j1) return;
    T L[9], R[9];
    face_states<T, DIR>(G, V, Vinit, i, j, k, Scal<T>::dt(sc), Scal<T>::psi(sc), L, R);
    long long nf = (long long)(G.ixmax - 1) * (G.jymax - 1) * (G.kzmax - 1);
    long long q = ((long long)i * (G.jymax - 1) + j) * (G.kzmax - 1) + k;
#pragma unroll
    for (int m = 0; m < 9; m++) { Vl[m * nf + q] = L[m]; Vr[m * nf + q] = R[m]; }
}

/* ------------------------------------------------------------------------ */
/* update + pointwise tail                                                   */
/* ------------------------------------------------------------------------ */

/* is cell (i,j,k) one that a boundary fill copies from? */
__device__ __forceinline__ bool is_bc_source(const Geom &G, int i, int j, int k)
{
    return i == 1 || i == G.ixmax - 2 || j == 1 || j == G.jymax - 2 || k == 1 || k == 2 || k == G.kzmax - 2;
}

/* absorbing layers after the boundary fills of the last stage:
 * XRightAbsorbBoundary (xboundary.h:133-138), CentralAbsorbBoundary
 * (centralboundary.h:36-41), ZRightAbsorbBoundary (zboundary.h:40-46, RK2 only) */
template <typename T>
__device__ __forceinline__ void absorb(const Geom &G, const T *__restrict__ Uinit, int i, int j, int k, bool zright,
                                      T u[9])
{
    const Tabs<T> &tb = tabs<T>(G);
    long long q = cidx(G, i, j, k);
    int ix0 = G.ixmax - 11, kz0 = G.kzmax - 11;
    bool ax = i >= ix0, ac = i <= G.irin, az = zright && k >= kz0;
    if (!(ax || ac || az)) return;
    T fx = ax ? tb.xabs[i - ix0] : T(0), fc = ac ? tb.cabs[(long long)i * G.kzmax + k] : T(0);
    T fz = az ? tb.zabs[k - kz0] : T(0);
#pragma unroll
    for (int m = 0; m < 9; m++) {
        T ui = Uinit[m * G.nc + q];
        T v = u[m];
        if (ax) v -= (fx * (v - ui));
        if (ac) v -= (fc * (v - ui));
        if (az) v -= (fz * (v - ui));
        u[m] = v;
    }
}

/* the six geometric factors of cell (i,k) (cylindricalgrid.h:120-125):
 * g[0..5] = g1..g6, weights of the lower/upper r, phi and z face fluxes */
template <typename T>
__device__ __forceinline__ void geo_factors(const Geom &G, int i, int k, T g[6])
{
    const Tabs<T> &tb = tabs<T>(G);
    const long long gk = (long long)i * G.kzmax + k, pl = (long long)G.ixmax * G.kzmax;
#pragma unroll
    for (int s = 0; s < 6; s++) g[s] = tb.g[s * pl + gk];
}

/* flux divergence of one variable from its six face fluxes, in the
 * reference's order (firststep.h:105-110) */
template <typename T>
__device__ __forceinline__ T flux_div(const T g[6], T fu, T fl, T gu, T gl, T hu, T hl)
{
    return ((g[1] * fu - g[0] * fl) + (g[3] * gu - g[2] * gl) + (g[5] * hu - g[4] * hl));
}

/* The k-plane ghost an interior cell (i,j,k) is the source of, if any (the
 * z fills: RK2 ZLeftVzAntisym / ZRightFree, k=0 <- k=2 with rho v_z negated
 * and kzmax-1 <- kzmax-2, zboundary.h:67-96,203-226; RK3 periodic, k=0 <-
 * kzmax-2 and kzmax-1 <- 1, zboundary.h:105-161), filled from the cell's raw
 * updated state u with the ghost's own pointwise tail -- the operations of
 * ghost_cell for that ghost, done while the source's row is in flight, so the
 * ghost kernel leaves these uncoalesced cells out.  Floor counts go straight
 * to the counters. */
template <typename T>
__device__ __forceinline__ void zghost_fill(const Geom &G, const StageArgs<T> &a, int i, int j, int k, const T u[9])
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
    const long long nc = G.nc, qg = cidx(G, i, j, kg);
    T ug[9], W[9];
#pragma unroll
    for (int m = 0; m < 9; m++) ug[m] = (flip && m == 3) ? -u[m] : u[m];
    if (a.last) absorb<T>(G, a.Uinit, i, j, kg, G.scheme == MHD_SCHEME_RK2, ug);
    const int flags = utov_check<T>(G, i, a.rhofloor[qg], ug, W);
    round_stored<T>(G, ug, W);
    T *Uo = (a.kind == 0 || a.kind == 1) ? a.U1 : a.Un;
#pragma unroll
    for (int m = 0; m < 9; m++) { Uo[m * nc + qg] = ug[m]; a.Vout[m * nc + qg] = W[m]; }
    if (flags & 1) atomicAdd(&a.counters[0], 1);
    if (flags & 2) atomicAdd(&a.counters[1], 1);
    if (flags & 4) atomicAdd(&a.counters[2], 1);
}

/* a cell's stage inputs read from global memory: V, U^n, U^(k), the floor */
template <typename T>
struct GmemCell {
    const StageArgs<T> &a;
    long long nc, q;
    __device__ __forceinline__ T v(int m) const { return a.V[m * nc + q]; }
    __device__ __forceinline__ T un(int m) const { return a.Un[m * nc + q]; }
    __device__ __forceinline__ T u1(int m) const { return a.U1[m * nc + q]; }
    __device__ __forceinline__ T rho() const { return a.rhofloor[q]; }
};

/* kind: 0 U1=U-dtL (Halfstep/FirstStep), 1 U1=(3U+U1-dtL)/4 (SecondStep),
 *       2 U=(U+2(U1-dtL))/3 (ThirdStep), 3 U=(U+U1-dtL)/2 (Fullstep)
 * div[] = the flux divergence of each variable at (i,j,k) (linear index q);
 * the cell's other inputs come through `in` (global memory, or a tile staged
 * in shared memory). */
template <typename T, typename In>
__device__ __forceinline__ int update_core(const Geom &G, const StageArgs<T> &a, int i, int j, int k, long long q,
                                           const T div[9], const In &in)
{
    const StepScalars *sc = a.sc;
    const long long nc = G.nc;
    const T dt = Scal<T>::dt(sc), psicoef = Scal<T>::psi(sc);
    const int kind = a.kind;
    T W[9], S[9], u[9];
    const StageCoef kc = stage_coef(kind);
    if (sizeof(T) == 4 && a.wfromu) {
        /* the stage's input primitives are UtoV of its input state U^(k)
         * (U^n in the first stage, U1 after it): recomputed, not loaded */
#pragma unroll
        for (int m = 0; m < 9; m++) u[m] = (kind == 0) ? in.un(m) : in.u1(m);
        utov<T>(G, i, u, W);
    } else {
#pragma unroll
        for (int m = 0; m < 9; m++) W[m] = in.v(m);
    }
    source_at<T>(G, *sc, a.trig, a.trigf, i, j, k, W, S);
#pragma unroll
    for (int m = 0; m < 9; m++) {
        T un = in.un(m), u1 = (kind == 0) ? T(0) : in.u1(m);
        T v;
        if (sizeof(T) == 4) {
            /* precision form: the combination in increment form (stage_combine_k) */
            if (m == 8) { un = psicoef * un; u1 = psicoef * u1; }   /* GLMSourceSolver on U and U1 */
            v = (T)stage_combine_k(kc, (float)un, (float)u1, (float)dt, (float)div[m], (float)S[m]);
        } else {
            if (m == 8) { un = psicoef * un; u1 = psicoef * u1; }   /* GLMSourceSolver on U and U1 */
            if (kind == 0) v = un - dt * div[m] + dt * S[m];
            else if (kind == 1) v = T(0.25) * (T(3.0) * un + u1 - dt * div[m] + dt * S[m]);
            else if (kind == 2) v = T(MHD_ONEO3) * (un + T(2.0) * (u1 - dt * div[m] + dt * S[m]));
            else v = T(0.5) * (un + u1 - dt * div[m] + dt * S[m]);
        }
        u[m] = v;
    }
    if (is_bc_source(G, i, j, k)) {
#pragma unroll
        for (int m = 0; m < 9; m++) a.Uraw[m * nc + q] = u[m];
        if (a.zghost) zghost_fill<T>(G, a, i, j, k, u);
    }
    if (G.scheme == MHD_SCHEME_RK2 && k == 1) u[3] = T(0.0);   /* zboundary.h:87 */
    if (a.last) absorb<T>(G, a.Uinit, i, j, k, G.scheme == MHD_SCHEME_RK2, u);
    int flags = utov_check<T>(G, i, in.rho(), u, W);
    round_stored<T>(G, u, W);
    T *Uo = (kind == 0 || kind == 1) ? a.U1 : a.Un;
#pragma unroll
    for (int m = 0; m < 9; m++) { Uo[m * nc + q] = u[m]; a.Vout[m * nc + q] = W[m]; }
    return flags;
}

template <typename T>
__device__ __forceinline__ int update_apply(const Geom &G, const StageArgs<T> &a, int i, int j, int k,
                                            const T div[9])
{
    const long long q = cidx(G, i, j, k);
    return update_core<T>(G, a, i, j, k, q, div, GmemCell<T>{a, G.nc, q});
}

/* update of one interior cell from the face fluxes in F/G/H */
template <typename T>
__device__ __forceinline__ int update_cell(const Geom &G, const StageArgs<T> &a, int i, int j, int k)
{
    const long long nc = G.nc, q = cidx(G, i, j, k);
    const long long si = (long long)G.jymax * G.kzmax, sj = G.kzmax;
    /* the upper z face of the last cell of a row from the compact Hb, where
     * the split stage keeps it */
    const T *hu = a.H + q;
    long long hs = nc;
    if (a.Hb && k == G.kzmax - 2) {
        hu = a.Hb + (long long)(i - 1) * (G.jymax - 2) + (j - 1);
        hs = (long long)(G.ixmax - 2) * (G.jymax - 2);
    }
    T g[6], div[9];
    geo_factors<T>(G, i, k, g);
#pragma unroll
    for (int m = 0; m < 9; m++) {
        const long long mq = m * nc + q;
        div[m] = flux_div<T>(g, a.F[mq], a.F[mq - si], a.G[mq], a.G[mq - sj], hu[m * hs], a.H[mq - 1]);
    }
    return update_apply<T>(G, a, i, j, k, div);
}

template <typename T>
__device__ __forceinline__ void prefetch_run(const T *p, long long n, long long e0, long long e1);

/* The update's streamed inputs of the block a.prefetch blocks ahead (in
 * launch order, about one wave of resident blocks), prefetched into L2 by
 * the first warp with bulk prefetches: V, F, G, H, U^n, U^(k) and the
 * density floor rows of that block's cells (the F and G rows one plane and
 * one row lower were prefetched for earlier blocks).  Each block then finds
 * its inputs in L2, so the DRAM reads run a wave ahead without holding
 * registers or shared memory. */
template <typename T>
__device__ __forceinline__ void update_prefetch_ahead(const Geom &G, const StageArgs<T> &a)
{
    const int lane = threadIdx.x + blockDim.x * threadIdx.y;
    if (lane >= 32) return;
    const long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
    const long long b = (long long)blockIdx.x + gridDim.x * ((long long)blockIdx.y + (long long)gridDim.y * blockIdx.z)
                        + a.prefetch;
    if (b >= nb) return;
    const int bx = (int)(b % gridDim.x), by = (int)((b / gridDim.x) % gridDim.y), bz = (int)(b / ((long long)gridDim.x * gridDim.y));
    const int k0 = 1 + bx * blockDim.x, i = a.ibeg + bz;
    const int kn = min((int)blockDim.x, G.kzmax - 1 - k0);
    const long long nc = G.nc, n9 = 9 * nc;
    for (int t = lane; t < 7 * (int)blockDim.y * 9; t += 32) {
        const int arr = t / (9 * blockDim.y), rem = t % (9 * blockDim.y), m = rem / blockDim.y;
        const int j = 1 + by * blockDim.y + rem % blockDim.y;
        if (j >= G.jymax - 1 || kn <= 0) continue;
        const long long q = cidx(G, i, j, k0) + m * nc;
        switch (arr) {
        case 0: prefetch_run<T>(a.V, n9, q, q + kn); break;
        case 1: prefetch_run<T>(a.F, n9, q, q + kn); break;
        case 2: prefetch_run<T>(a.G, n9, q, q + kn); break;
        case 3: prefetch_run<T>(a.H, n9, q - 1, q + kn); break;
        case 4: prefetch_run<T>(a.Un, n9, q, q + kn); break;
        case 5: if (a.kind != 0) prefetch_run<T>(a.U1, n9, q, q + kn); break;
        default: if (m == 0) prefetch_run<T>(a.rhofloor, nc, q, q + kn); break;
        }
    }
}

/* FP32: 9 resident blocks of 128 threads per SM (56 registers, 4 bytes
 * spilled): 3.32 ms per launch at 512x512x256 against 3.42 ms at 8 blocks
 * (64 registers), 3.40 at 10 (48) and 3.92 at 12 (40) -- the kernel waits on
 * memory, and the ninth block keeps more loads in flight. */
template <typename T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 9 : 1) update_kernel(Geom G, StageArgs<T> a)
{
    if (a.sc->dtbad) return;
    if (a.prefetch) update_prefetch_ahead<T>(G, a);
    const int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = a.ibeg + blockIdx.z;
    int flags = 0;
    if (k < G.kzmax - 1 && j < G.jymax - 1) flags = update_cell<T>(G, a, i, j, k);
    add_counters(flags, a.counters);
}

/* ------------------------------------------------------------------------ */
/* TMA-staged update (precision form)                                        */
/* ------------------------------------------------------------------------ */
/* One block per tile of MHD_UPD_TILE consecutive cells of the flat [i][j][k]
 * index.  One thread loads the tile's inputs into shared memory with tensor
 * copies (cp.async.bulk.tensor, completing on an mbarrier): V, F, G, U^n,
 * U^(k), the floor at the tile, and F, G, H at the tile shifted by one plane,
 * one row and one cell (windows MHD_UPD_WIDE wide from the 16-byte boundary at
 * or before the shifted start).  The loads hold no registers, so each SM keeps
 * several tiles (about 40 KB each) in flight; the update itself is
 * update_core, one thread per cell, ghost cells skipped.  The wait is bounded:
 * a tile whose copies do not land within `spin` polls sets *err, waits as long
 * again for the copies still in flight and leaves the tile untouched.  Should
 * that second wait run out as well, the block exits while bulk copies may
 * still be writing its shared memory -- unsafe, which is one reason this path
 * is an option that stays off, and no test drives either wait to its limit.
 * Measured at 512x512x256: 3.62 ms per launch against 3.38 ms for
 * update_kernel (3.69 ms with all on-chip memory as shared memory): five
 * 38 KB tiles per SM keep more bytes in flight than the thread loads, but
 * each block then computes with 4 warps and 20 per SM instead of 32, and the
 * update's arithmetic (sources, the FP64 pressure repair) no longer hides
 * under other warps' loads.  An option (mhd_set_update_path); the thread
 * loads stay the default. */
struct UpdTile {
    alignas(128) float v[9 * MHD_UPD_TILE];
    alignas(128) float f[9 * MHD_UPD_TILE];
    alignas(128) float g[9 * MHD_UPD_TILE];
    alignas(128) float un[9 * MHD_UPD_TILE];
    alignas(128) float u1[9 * MHD_UPD_TILE];
    alignas(128) float fm[9 * MHD_UPD_WIDE];
    alignas(128) float gm[9 * MHD_UPD_WIDE];
    alignas(128) float h[9 * MHD_UPD_WIDE];
    alignas(128) float rho[MHD_UPD_TILE];
    alignas(8) unsigned long long bar;
};

/* a cell's stage inputs from the staged tile (t = the cell's slot) */
struct TileCell {
    const UpdTile &s;
    int t;
    __device__ __forceinline__ float v(int m) const { return s.v[m * MHD_UPD_TILE + t]; }
    __device__ __forceinline__ float un(int m) const { return s.un[m * MHD_UPD_TILE + t]; }
    __device__ __forceinline__ float u1(int m) const { return s.u1[m * MHD_UPD_TILE + t]; }
    __device__ __forceinline__ float rho() const { return s.rho[t]; }
};

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];"
                 :: "r"(smem_addr(dst)), "l"((unsigned long long)map), "r"(x), "r"(y), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned phase)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_addr(bar)), "r"(phase) : "memory");
    return ok != 0;
}

template <typename T>
__global__ void __launch_bounds__(MHD_UPD_TILE)
update_tma_kernel(Geom G, StageArgs<T> a, const __grid_constant__ UpdMaps maps, int vpar, long long qbeg,
                  int *err, int spin)
{
    static_assert(sizeof(T) == 4, "the staged tile holds FP32 state");
    __shared__ UpdTile s;
    if (a.sc->dtbad) return;
    const long long q0 = qbeg + (long long)blockIdx.x * MHD_UPD_TILE;
    const long long si = (long long)G.jymax * G.kzmax, sj = G.kzmax;
    const int xfm = (int)((q0 - si) & ~3LL), xgm = (int)((q0 - sj) & ~3LL), xh = (int)((q0 - 1) & ~3LL);
    const int x0 = (int)q0;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&s.bar)) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned narrow = 9 * MHD_UPD_TILE * 4, wide = 9 * MHD_UPD_WIDE * 4;
        const unsigned bytes = (a.kind != 0 ? 5 : 4) * narrow + 3 * wide + MHD_UPD_TILE * 4;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                     :: "r"(smem_addr(&s.bar)), "r"(bytes) : "memory");
        tma_load_2d(s.v, &maps.v[vpar], x0, 0, &s.bar);
        tma_load_2d(s.f, &maps.f, x0, 0, &s.bar);
        tma_load_2d(s.g, &maps.g, x0, 0, &s.bar);
        tma_load_2d(s.un, &maps.un, x0, 0, &s.bar);
        if (a.kind != 0) tma_load_2d(s.u1, &maps.u1, x0, 0, &s.bar);
        tma_load_2d(s.fm, &maps.fm, xfm, 0, &s.bar);
        tma_load_2d(s.gm, &maps.gm, xgm, 0, &s.bar);
        tma_load_2d(s.h, &maps.h, xh, 0, &s.bar);
        tma_load_2d(s.rho, &maps.rho, x0, 0, &s.bar);
    }
    bool ok = false;
    for (int it = 0; it < spin && !ok; it++) ok = mbar_try_wait(&s.bar, 0);
    if (!__syncthreads_and(ok)) {   /* the whole block leaves together */
        if (threadIdx.x == 0) atomicExch(err, 1);
        for (int it = 0; it < spin && !ok; it++) ok = mbar_try_wait(&s.bar, 0);
        return;
    }
    const int t = threadIdx.x;
    const long long q = q0 + t;
    const int k = (int)(q % G.kzmax);
    const long long r = q / G.kzmax;
    const int j = (int)(r % G.jymax), i = (int)(r / G.jymax);
    int flags = 0;
    if (i >= 1 && i <= G.ixmax - 2 && j >= 1 && j <= G.jymax - 2 && k >= 1 && k <= G.kzmax - 2) {
        const int of = (int)(q - si) - xfm, og = (int)(q - sj) - xgm, oh = (int)(q - 1) - xh;
        float gg[6], div[9];
        geo_factors<float>(G, i, k, gg);
#pragma unroll
        for (int m = 0; m < 9; m++)
            div[m] = flux_div<float>(gg, s.f[m * MHD_UPD_TILE + t], s.fm[m * MHD_UPD_WIDE + of],
                                     s.g[m * MHD_UPD_TILE + t], s.gm[m * MHD_UPD_WIDE + og],
                                     s.h[m * MHD_UPD_WIDE + oh + 1], s.h[m * MHD_UPD_WIDE + oh]);
        flags = update_core<float>(G, a, i, j, k, q, div, TileCell{s, t});
    }
    add_counters(flags, a.counters);
}

/* ------------------------------------------------------------------------ */
/* fused stage: fluxes and update of the interior in one kernel              */
/* ------------------------------------------------------------------------ */
/* Riemann + GLM flux of face (i,j,k) along DIR (face index convention of
 * flux_face: face f lies between cells f and f+1) into Fo */
template <typename T, int DIR>
__device__ __forceinline__ void face_flux_at(const Geom &G, const T *__restrict__ V, const T *__restrict__ Vinit,
                                             const StepScalars *__restrict__ sc, int i, int j, int k, T Fo[9])
{
    T dt = Scal<T>::dt(sc), ch = Scal<T>::ch(sc), psicoef = Scal<T>::psi(sc);
    T L[9], R[9];
    face_states<T, DIR>(G, V, Vinit, i, j, k, dt, psicoef, L, R);
    face_flux<T, DIR>(G, L, R, i, ch, Fo);
}

/* z fluxes and the update in one kernel, with no block barrier.  A warp owns
 * ROWS rows (i, j) of cells and walks each in chunks of 32 cells along k:
 * lane l forms the z flux of the upper face of cell k0 + l into the warp's
 * row of shared memory, whose slot 0 carries the previous chunk's last face,
 * so the lower face of every cell is its neighbour's slot.  The
 * two boundary faces of each row (face 0, with its antisymmetric / fixed /
 * periodic left state, and face kzmax-2) are formed first for all ROWS rows at
 * once and kept in shared memory, so no chunk diverges on them.  Each lane
 * then updates its cell from the r and phi fluxes in F, G and its z fluxes in
 * registers: the z fluxes never reach HBM and the update's loads overlap other
 * warps' flux arithmetic.  Same operations as the split z flux followed by
 * update_kernel<T>, so the plain form keeps its bits.  Measured at
 * 512x512x256 (FP32): 6.3 ms against 1.9 + 3.4 ms for the two kernels apart
 * (at 128 registers 8.5 ms, 80 registers 6.8 ms; an L2 prefetch of each
 * chunk's inputs made it slower); the split kernels stay the default. */
template <typename T, int ROWS>
__global__ void __launch_bounds__(128, 8) zupdate_kernel(Geom G, StageArgs<T> a)
{
    if (a.sc->dtbad) return;
    __shared__ T sedge[4][2][9][ROWS];
    __shared__ T sh[4][9][33];   /* per warp: slot s = z face k0 - 1 + s of the current chunk */
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nj = G.jymax - 2, kz = G.kzmax - 2, klast = G.kzmax - 2;
    const long long nrow = (long long)(G.ixmax - 2) * nj;
    const long long row0 = ((long long)blockIdx.x * 4 + w) * ROWS;
    if (row0 >= nrow) return;   /* a whole warp: no shuffle partner left behind */
    const T *__restrict__ V = a.V;
    const T *__restrict__ Vinit = a.Vinit;
    const StepScalars *__restrict__ sc = a.sc;
    /* the boundary faces of the warp's rows: lane l < ROWS face 0 of row l,
     * ROWS <= l < 2 ROWS face kzmax-2 of row l - ROWS */
    if (lane < 2 * ROWS) {
        const int rr = lane < ROWS ? lane : lane - ROWS;
        const long long r = row0 + rr;
        if (r < nrow) {
            const int i = 1 + (int)(r / nj), j = 1 + (int)(r % nj);
            T f[9];
            face_flux_at<T, 2>(G, V, Vinit, sc, i, j, lane < ROWS ? 0 : klast, f);
#pragma unroll
            for (int m = 0; m < 9; m++) sedge[w][lane < ROWS ? 0 : 1][m][rr] = f[m];
        }
    }
    __syncwarp();
    const long long nc = G.nc, si = (long long)G.jymax * G.kzmax, sj = G.kzmax;
    unsigned c0 = 0, c1 = 0, c2 = 0;
    for (int rr = 0; rr < ROWS; rr++) {
        const long long r = row0 + rr;
        if (r >= nrow) break;   /* warp-uniform */
        const int i = 1 + (int)(r / nj), j = 1 + (int)(r % nj);
        if (lane < 9) sh[w][lane][0] = sedge[w][0][lane][rr];
        __syncwarp();
        for (int k0 = 1; k0 <= kz; k0 += 32) {
            const int k = k0 + lane;
            const bool live = k <= kz;
            {
                T hu[9];
                if (!live) {
#pragma unroll
                    for (int m = 0; m < 9; m++) hu[m] = T(0.0);
                } else if (k == klast) {
#pragma unroll
                    for (int m = 0; m < 9; m++) hu[m] = sedge[w][1][m][rr];
                } else {
                    face_flux_at<T, 2>(G, V, Vinit, sc, i, j, k, hu);
                }
#pragma unroll
                for (int m = 0; m < 9; m++) sh[w][m][lane + 1] = hu[m];
            }
            __syncwarp();
            if (live) {
                const long long q = cidx(G, i, j, k);
                T g[6], div[9];
                geo_factors<T>(G, i, k, g);
#pragma unroll
                for (int m = 0; m < 9; m++) {
                    const long long mq = m * nc + q;
                    div[m] = flux_div<T>(g, a.F[mq], a.F[mq - si], a.G[mq], a.G[mq - sj], sh[w][m][lane + 1],
                                         sh[w][m][lane]);
                }
                int flags = update_apply<T>(G, a, i, j, k, div);
                c0 += flags & 1; c1 += (flags >> 1) & 1; c2 += (flags >> 2) & 1;
            }
            __syncwarp();
            if (lane < 9) sh[w][lane][0] = sh[w][lane][32];   /* the carry into the next chunk */
            __syncwarp();
        }
    }
    add_counts3(c0, c1, c2, a.counters);
}

/* L2 prefetch of the bytes of elements [e0, e1) of array p (n elements) through
 * the bulk-copy unit: one instruction per contiguous run.  The range is clipped
 * to the array and to 16-byte boundaries inside it (the array base is
 * 256-byte aligned), so no byte outside the allocation is named. */
template <typename T>
__device__ __forceinline__ void prefetch_run(const T *p, long long n, long long e0, long long e1)
{
    if (e0 < 0) e0 = 0;
    if (e1 > n) e1 = n;
    if (e1 <= e0) return;
    unsigned long long s = (unsigned long long)(p + e0) & ~15ull;
    unsigned long long e = (unsigned long long)(p + e1) & ~15ull;
    if (e > s)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(s), "r"((unsigned)(e - s)) : "memory");
}

/* One block = a tile of 32 (k) x TJ (j) cells marching over a run of seg
 * planes in i, with TJ + 1 warps: warp w >= 1 owns row j0 + w - 1, warp 0
 * is the tile's helper.  Per plane each row warp forms the r, phi and z
 * fluxes of its cells' upper faces (three face rounds); the helper forms the
 * tile's lower phi faces (one round) and lower z faces (one partial round)
 * and issues the L2 prefetches of the next plane's inputs, so every warp's
 * path to the barrier is at most three rounds.  The r flux of a cell's lower
 * face is the previous plane's upper one.  The face fluxes meet in shared
 * memory (double-buffered by plane, so one barrier per plane suffices) and
 * never travel to HBM; every face of the stage is computed once, plus one r
 * face per run and the tile's edge faces.  The update, sources, UtoV and
 * Check follow in the same thread: one launch replaces the flux(r),
 * flux(phi), flux(z) and update kernels. */
template <typename T, int TJ>
struct StageSmem {
    T fr[2][TJ][9][32];        /* r fluxes of the lower / upper face, ping-pong by plane */
    T fg[2][TJ + 1][9][32];    /* phi faces: [plane parity][s] = face j0 + s - 1 */
    T fh[2][TJ][9][33];        /* z faces: [plane parity][row][s] = face k0 + s - 1 */
};

template <typename T, int TJ, int MINB>
__global__ void __launch_bounds__(32 * (TJ + 1), MINB) stage_kernel(Geom G, StageArgs<T> a, int seg)
{
    if (a.sc->dtbad) return;
    extern __shared__ __align__(16) unsigned char stage_smem_raw[];
    StageSmem<T, TJ> &sm = *reinterpret_cast<StageSmem<T, TJ> *>(stage_smem_raw);
    const int lane = threadIdx.x, w = threadIdx.y, jj = w - 1;
    const int k0 = 1 + blockIdx.x * 32, j0 = 1 + blockIdx.y * TJ;
    const int k = k0 + lane, j = j0 + jj;
    const int ia = 1 + blockIdx.z * seg;
    const int ib = min(ia + seg, G.ixmax - 1);
    const bool kin = k < G.kzmax - 1;
    const bool live = w > 0 && kin && j < G.jymax - 1;
    const T *__restrict__ V = a.V;
    const T *__restrict__ Vinit = a.Vinit;
    const StepScalars *__restrict__ sc = a.sc;
    const long long nc = G.nc, nall = 9 * nc, si = (long long)G.jymax * G.kzmax;
    unsigned c0 = 0, c1 = 0, c2 = 0;
    T f[9];
    if (live) {
        face_flux_at<T, 0>(G, V, Vinit, sc, ia - 1, j, k, f);
#pragma unroll
        for (int m = 0; m < 9; m++) sm.fr[0][jj][m][lane] = f[m];
    }
    int lo = 0, b = 0;
    for (int i = ia; i < ib; i++) {
        if (w > 0) {
            if (live) {
                face_flux_at<T, 0>(G, V, Vinit, sc, i, j, k, f);
#pragma unroll
                for (int m = 0; m < 9; m++) sm.fr[lo ^ 1][jj][m][lane] = f[m];
                face_flux_at<T, 1>(G, V, Vinit, sc, i, j, k, f);
#pragma unroll
                for (int m = 0; m < 9; m++) sm.fg[b][jj + 1][m][lane] = f[m];
                face_flux_at<T, 2>(G, V, Vinit, sc, i, j, k, f);
#pragma unroll
                for (int m = 0; m < 9; m++) sm.fh[b][jj][m][lane + 1] = f[m];
            }
        } else {
            /* next plane's cold inputs: U^n, U^(k), rhofloor rows of the
             * tile, and the V plane the r reconstruction reaches next */
            if (i + 1 < ib) {
                const long long row0 = ((long long)(i + 1) * G.jymax + j0) * G.kzmax + k0;
                for (int t = lane; t < 19 * TJ; t += 32) {
                    const int v = t / TJ, r = t - v * TJ;
                    if (j0 + r >= G.jymax - 1) continue;
                    const long long e0 = row0 + (long long)r * G.kzmax;
                    if (v < 9) prefetch_run<T>(a.Un, nall, v * nc + e0, v * nc + e0 + 32);
                    else if (v < 18) { if (a.kind != 0) prefetch_run<T>(a.U1, nall, (v - 9) * nc + e0, (v - 9) * nc + e0 + 32); }
                    else prefetch_run<T>(a.rhofloor, nc, e0, e0 + 32);
                }
            }
            if (i + 3 < G.ixmax) {
                const long long pl0 = (long long)(i + 3) * si;
                for (int t = lane; t < 9 * (TJ + 4); t += 32) {
                    const int v = t / (TJ + 4), jr = j0 - 2 + (t - v * (TJ + 4));
                    if (jr < 0 || jr >= G.jymax) continue;
                    const long long e0 = v * nc + pl0 + (long long)jr * G.kzmax;
                    const int ka = max(k0 - 2, 0), kb = min(k0 + 34, G.kzmax);
                    prefetch_run<T>(V, nall, e0 + ka, e0 + kb);
                }
            }
            if (kin && j0 < G.jymax - 1) {
                face_flux_at<T, 1>(G, V, Vinit, sc, i, j0 - 1, k, f);
#pragma unroll
                for (int m = 0; m < 9; m++) sm.fg[b][0][m][lane] = f[m];
            }
            if (lane < TJ && j0 + lane < G.jymax - 1 && k0 < G.kzmax - 1) {
                face_flux_at<T, 2>(G, V, Vinit, sc, i, j0 + lane, k0 - 1, f);
#pragma unroll
                for (int m = 0; m < 9; m++) sm.fh[b][lane][m][0] = f[m];
            }
        }
        __syncthreads();
        if (live) {
            T g[6], div[9];
            geo_factors<T>(G, i, k, g);
#pragma unroll
            for (int m = 0; m < 9; m++)
                div[m] = flux_div<T>(g, sm.fr[lo ^ 1][jj][m][lane], sm.fr[lo][jj][m][lane], sm.fg[b][jj + 1][m][lane],
                                     sm.fg[b][jj][m][lane], sm.fh[b][jj][m][lane + 1], sm.fh[b][jj][m][lane]);
            int flags = update_apply<T>(G, a, i, j, k, div);
            c0 += flags & 1; c1 += (flags >> 1) & 1; c2 += (flags >> 2) & 1;
        }
        lo ^= 1;
        b ^= 1;
    }
    add_counts3(c0, c1, c2, a.counters);
}

/* Ghost cell -> (source interior cell, sign flip mask) after the fill sequence
 * Y periodic (yboundary.h:97-154), X axis (xboundary.h:33-72), X right free
 * (xboundary.h:322-346), then Z: RK2 k=0 antisymmetric in v_z and k=kzmax-1
 * free (zboundary.h:67-96,203-226); RK3 periodic (zboundary.h:105-161).
 * Later fills win, so the map is applied Z first, then X, then Y. */
__device__ __forceinline__ void ghost_source(const Geom &G, int i, int j, int k, int &si, int &sj, int &sk,
                                             unsigned &neg)
{
    neg = 0u;
    sk = k;
    if (G.scheme == MHD_SCHEME_RK2) {
        if (k == 0) { sk = 2; neg ^= 1u << 3; }
        else if (k == G.kzmax - 1) sk = G.kzmax - 2;
    } else {
        if (k == 0) sk = G.kzmax - 2;
        else if (k == G.kzmax - 1) sk = 1;
    }
    si = i; sj = j;
    int half = G.jy / 2;
    if (i == 0) {
        si = 1;
        sj = (j < half + 1) ? j + half : j - half;
        neg ^= (1u << 1) | (1u << 2) | (1u << 4) | (1u << 5);
        return;   /* the axis source row j' is always interior */
    }
    if (i == G.ixmax - 1) si = G.ixmax - 2;
    if (j == 0) sj = G.jymax - 2;
    else if (j == G.jymax - 1) sj = 1;
}

/* number of ghost cells and the ghost cell with enumeration index tid:
 * k planes (k=0, kzmax-1), then j planes, then i planes.  zg = 1: of the k
 * planes only the rim (i or j a ghost index); the update fills the rest */
__host__ __device__ __forceinline__ unsigned ghost_kplane(unsigned ni, unsigned nj, int zg)
{
    return zg ? 2 * nj + 2 * (ni - 2) : ni * nj;
}

__host__ __device__ __forceinline__ unsigned ghost_count(const Geom &G, int zg = 0)
{
    const unsigned nk = G.kzmax, nj = G.jymax, ni = G.ixmax;
    return 2 * ghost_kplane(ni, nj, zg) + 2 * ni * (nk - 2) + 2 * (nj - 2) * (nk - 2);
}

__device__ __forceinline__ void ghost_cell_of(const Geom &G, unsigned tid, int zg, int &i, int &j, int &k)
{
    const unsigned nk = G.kzmax, nj = G.jymax, ni = G.ixmax;
    const unsigned kp = ghost_kplane(ni, nj, zg);
    const unsigned nkplane = 2 * kp;
    const unsigned njplane = 2 * ni * (nk - 2);
    if (tid < nkplane) {
        k = (tid < kp) ? 0 : (int)nk - 1;
        unsigned r = tid % kp;
        if (!zg) {
            i = (int)(r / nj); j = (int)(r % nj);
        } else if (r < 2 * nj) {
            i = (r < nj) ? 0 : (int)ni - 1; j = (int)(r % nj);
        } else {
            r -= 2 * nj;
            j = (r < ni - 2) ? 0 : (int)nj - 1; i = 1 + (int)(r % (ni - 2));
        }
    } else if (tid < nkplane + njplane) {
        unsigned r = tid - nkplane;
        j = (r < ni * (nk - 2)) ? 0 : (int)nj - 1;
        r %= ni * (nk - 2);
        i = (int)(r / (nk - 2)); k = 1 + (int)(r % (nk - 2));
    } else {
        unsigned r = tid - nkplane - njplane;
        i = (r < (nj - 2) * (nk - 2)) ? 0 : (int)ni - 1;
        r %= (nj - 2) * (nk - 2);
        j = 1 + (int)(r / (nk - 2)); k = 1 + (int)(r % (nk - 2));
    }
}

template <typename T>
__device__ __forceinline__ int ghost_cell(const Geom &G, const StageArgs<T> &a, unsigned tid)
{
    int i, j, k;
    ghost_cell_of(G, tid, a.zghost, i, j, k);
    int si, sj, sk;
    unsigned neg;
    ghost_source(G, i, j, k, si, sj, sk, neg);
    const long long nc = G.nc, q = cidx(G, i, j, k), qs = cidx(G, si, sj, sk);
    T u[9], W[9];
#pragma unroll
    for (int m = 0; m < 9; m++) {
        T v = a.Uraw[m * nc + qs];
        u[m] = ((neg >> m) & 1u) ? -v : v;
    }
    if (G.scheme == MHD_SCHEME_RK2 && k == 1) u[3] = T(0.0);
    if (a.last) absorb<T>(G, a.Uinit, i, j, k, G.scheme == MHD_SCHEME_RK2, u);
    int flags = utov_check<T>(G, i, a.rhofloor[q], u, W);
    round_stored<T>(G, u, W);
    T *Uo = (a.kind == 0 || a.kind == 1) ? a.U1 : a.Un;
#pragma unroll
    for (int m = 0; m < 9; m++) { Uo[m * nc + q] = u[m]; a.Vout[m * nc + q] = W[m]; }
    return flags;
}

template <typename T>
__global__ void __launch_bounds__(128) ghost_kernel(Geom G, StageArgs<T> a)
{
    if (a.sc->dtbad) return;
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    int flags = 0;
    if (tid < ghost_count(G, a.zghost)) flags = ghost_cell<T>(G, a, tid);
    add_counters(flags, a.counters);
}

/* ------------------------------------------------------------------------ */
/* CFL reduction (setdt.h:33-89), always FP64                                */
/* ------------------------------------------------------------------------ */
__device__ __forceinline__ MaxLoc better(MaxLoc a, MaxLoc b)
{
    /* larger value wins; equal values: the smaller cell index (the serial
     * reference keeps the first cell reaching the maximum: strict '>') */
    if (b.q < 0) return a;
    if (a.q < 0) return b;
    if (b.v > a.v || (b.v == a.v && b.q < a.q)) return b;
    return a;
}

/* the CFL rate of one cell in FP64 (setdt.h:42-56) */
template <typename T>
__device__ __forceinline__ double cfl_rate64(const Geom &G, const T *__restrict__ V, int i, long long q, int k)
{
    const long long nc = G.nc;
    double v0 = V[q], v1 = V[nc + q], v2v = V[2 * nc + q], v3 = V[3 * nc + q];
    double v4 = V[4 * nc + q], v5 = V[5 * nc + q], v6 = V[6 * nc + q], v7 = V[7 * nc + q];
    double v2 = v1 * v1 + v2v * v2v + v3 * v3;
    double b2 = v4 * v4 + v5 * v5 + v6 * v6;
    double t1 = sqrt(v2 + (MHD_GM * v7 + b2) / v0) / G.minlength[(long long)i * G.kzmax + k];
    int cl = G.cooling ? cooling_rate(v0, v7) : 0;
    double tc = (2.0 * ((v0 * v0 * cl) / (1.5 * v7)));
    return rmax<double>(t1, tc);
}

/* The precision form's CFL rate of one cell in FP64: cfl_rate64 except that
 * a NaN rate (an invalid state) counts as infinite, so dt becomes 0 and the
 * dt guard stops the run at once.  The plain form keeps the reference's
 * semantics, where a NaN rate never wins (max() and the comparison of
 * setdt.h:57,60 are false for NaN). */
template <typename T>
__device__ __forceinline__ double cfl_rate64_strict(const Geom &G, const T *__restrict__ V, int i, long long q,
                                                    int k)
{
    const long long nc = G.nc;
    double v0 = V[q], v1 = V[nc + q], v2v = V[2 * nc + q], v3 = V[3 * nc + q];
    double v4 = V[4 * nc + q], v5 = V[5 * nc + q], v6 = V[6 * nc + q], v7 = V[7 * nc + q];
    double v2 = v1 * v1 + v2v * v2v + v3 * v3;
    double b2 = v4 * v4 + v5 * v5 + v6 * v6;
    double t1 = sqrt(v2 + (MHD_GM * v7 + b2) / v0) / G.minlength[(long long)i * G.kzmax + k];
    int cl = G.cooling ? cooling_rate(v0, v7) : 0;
    double tc = (2.0 * ((v0 * v0 * cl) / (1.5 * v7)));
    if (t1 != t1 || tc != tc) return INFINITY;
    return rmax<double>(t1, tc);
}

/* Plain form: every cell in FP64, bit-identical to setdt.h.  Precision form:
 * cells are screened in FP32 and each block's winner is re-evaluated in FP64,
 * so the maximum (and dt) carries FP64 rounding of an FP32-selected cell; a
 * cell whose rate is NaN wins with an infinite rate (dt = 0: the guard). */
template <typename T>
__global__ void __launch_bounds__(256)
setdt_kernel(Geom G, const T *__restrict__ V, MaxLoc *part)
{
    __shared__ MaxLoc sm[8];
    const int nj = G.jymax - 2;
    const int rows = (G.ixmax - 12) * nj;   /* i in [1, ixmax-11) (setdt.h:33) */
    MaxLoc best = {0.0, -1};
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int i = 1 + r / nj, j = 1 + r % nj;
        for (int k = 1 + threadIdx.x; k < G.kzmax - 1; k += blockDim.x) {
            const long long q = cidx(G, i, j, k);
            double tmp;
            if (sizeof(T) == 8) {
                tmp = cfl_rate64<T>(G, V, i, q, k);
            } else {
                const long long nc = G.nc;
                float v0 = V[q], v1 = V[nc + q], v2v = V[2 * nc + q], v3 = V[3 * nc + q];
                float v4 = V[4 * nc + q], v5 = V[5 * nc + q], v6 = V[6 * nc + q], v7 = V[7 * nc + q];
                float v2 = v1 * v1 + v2v * v2v + v3 * v3;
                float b2 = v4 * v4 + v5 * v5 + v6 * v6;
                float t1 = sqrtf(v2 + ((float)MHD_GM * v7 + b2) / v0) / (float)G.f.minlength[(long long)i * G.kzmax + k];
                int cl = G.cooling ? cooling_rate_f(v0, v7) : 0;
                float tc = (2.0f * ((v0 * v0 * (float)cl) / (1.5f * v7)));
                tmp = (t1 != t1 || tc != tc) ? (double)INFINITY : (double)rmax<float>(t1, tc);
            }
            /* the reference only takes a cell when its rate exceeds the running max (from 0) */
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
        if (sizeof(T) == 4 && b.q >= 0) {
            const int k = (int)(b.q % G.kzmax), i = (int)(b.q / ((long long)G.kzmax * G.jymax));
            b.v = cfl_rate64_strict<T>(G, V, i, b.q, k);
        }
        part[blockIdx.x] = b;
    }
}

/* ------------------------------------------------------------------------ */
/* conversions                                                               */
/* ------------------------------------------------------------------------ */
template <typename T>
__global__ void cvt_from_f64(const double *__restrict__ src, T *__restrict__ dst, long long n)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (T)src[t];
}

template <typename T>
__global__ void cvt_to_f64(const T *__restrict__ src, double *__restrict__ dst, long long n)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (double)src[t];
}

/* V = UtoV(U) at every cell, ghosts included (utov.h:24-68, no floors): the
 * primitives of a state uploaded without them */
template <typename T>
__global__ void __launch_bounds__(256) derive_v_kernel(Geom G, const T *__restrict__ U, T *__restrict__ V)
{
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < G.nc;
         q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q / ((long long)G.jymax * G.kzmax));
        T u[9], w[9];
#pragma unroll
        for (int m = 0; m < 9; m++) u[m] = U[m * G.nc + q];
        utov<T>(G, i, u, w);
#pragma unroll
        for (int m = 0; m < 9; m++) V[m * G.nc + q] = w[m];
    }
}

/* source term probe (SpiralGravityCooling over all cells) */
template <typename T>
__global__ void source_kernel(Geom G, const T *__restrict__ V, const StepScalars *__restrict__ sc,
                              const double *__restrict__ trig, const float *__restrict__ trigf,
                              double *__restrict__ S)
{
    long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= G.nc) return;
    int k = (int)(tid % G.kzmax);
    long long r = tid / G.kzmax;
    int j = (int)(r % G.jymax);
    int i = (int)(r / G.jymax);
    T W[9], Sv[9];
#pragma unroll
    for (int m = 0; m < 9; m++) W[m] = V[m * G.nc + tid];
    source_at<T>(G, *sc, trig, trigf, i, j, k, W, Sv);
#pragma unroll
    for (int m = 0; m < 9; m++) S[m * G.nc + tid] = (double)Sv[m];
}

/* ------------------------------------------------------------------------ */
/* launchers                                                                 */
/* ------------------------------------------------------------------------ */
static inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

/* SMs of the current device (152 on GB300), read once */
static inline int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            n = v;
        else
            n = 152;
    }
    return n;
}

/* 128-thread blocks laid along k (fastest index), rows of j stacked when the
 * k extent is short; one grid z-slice per i */
static inline void grid3(int nk, int nj, int ni, dim3 &grid, dim3 &block)
{
    int bx = 32 * ((nk + 31) / 32);
    if (bx > 128) bx = 128;
    int by = 128 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((nk + bx - 1) / bx, (nj + by - 1) / by, ni);
}

/* the z boundary faces (face 0 and kzmax-2) of a face box, if it has them */
static inline void zedge_sides(const Geom &G, const Box &b, int &lo, int &hi)
{
    lo = b.k0 == 0;
    hi = b.k1 > G.kzmax - 2 && b.k0 <= G.kzmax - 2 && G.kzmax - 2 > 0;
}

template <typename T>
cudaError_t launch_zedge_t(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F, Box b,
                           bool reflayout, cudaStream_t st)
{
    if (b.i1 <= b.i0 || b.j1 <= b.j0 || b.k1 <= b.k0) return cudaSuccess;
    int lo, hi;
    zedge_sides(G, b, lo, hi);
    if (!lo && !hi) return cudaSuccess;
    long long n = (long long)(b.i1 - b.i0) * (b.j1 - b.j0) * (lo + hi);
    if (reflayout) flux_zedge_kernel<T, true><<<nblocks(n, 128), 128, 0, st>>>(G, V, Vinit, sc, F, b, lo, hi);
    else flux_zedge_kernel<T, false><<<nblocks(n, 128), 128, 0, st>>>(G, V, Vinit, sc, F, b, lo, hi);
    return cudaGetLastError();
}

/* the split stage's z faces: the row walk (the interior faces, and the
 * boundary faces' slots into the scratch Zs, 27 values per (i,j) row);
 * needs at least two interior cells along z */
template <typename T>
cudaError_t launch_flux_zwalk_t(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F, T *Zs,
                                cudaStream_t st)
{
    const long long nrow = (long long)(G.ixmax - 2) * (G.jymax - 2);
    if (G.kzmax < 4) return cudaErrorInvalidValue;
    if (nrow <= 0) return cudaSuccess;
    Box b;
    b.i0 = 1; b.i1 = G.ixmax - 1; b.j0 = 1; b.j1 = G.jymax - 1; b.k0 = 0; b.k1 = G.kzmax - 1;
    zwalk_edges_kernel<T><<<nblocks(nrow, 4), 128, 0, st>>>(G, V, Vinit, sc, F, Zs, b);
    return cudaGetLastError();
}

/* ... and the last face of each row from that scratch, into Hb (and H with
 * Hfull) */
template <typename T>
cudaError_t launch_flux_zlast_t(const Geom &G, const T *Vinit, const StepScalars *sc, T *H, T *Hb, const T *Zs,
                                int Hfull, cudaStream_t st)
{
    const long long nrow = (long long)(G.ixmax - 2) * (G.jymax - 2);
    if (nrow <= 0) return cudaSuccess;
    zlast_flux_kernel<T><<<nblocks(nrow, 128), 128, 0, st>>>(G, Vinit, sc, H, Hb, Zs, Hfull);
    return cudaGetLastError();
}

/* dir 2 with edges = false leaves the boundary z faces to launch_zedge_t */
template <typename T>
cudaError_t launch_flux_t(int dir, const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F,
                          Box b, bool reflayout, cudaStream_t st, bool edges = true)
{
    if (b.i1 <= b.i0 || b.j1 <= b.j0 || b.k1 <= b.k0) return cudaSuccess;
    if (dir == 2) {
        /* boundary z faces in their own launch, the rest below */
        int lo, hi;
        zedge_sides(G, b, lo, hi);
        if (edges && (lo || hi)) {
            cudaError_t e = launch_zedge_t<T>(G, V, Vinit, sc, F, b, reflayout, st);
            if (e != cudaSuccess) return e;
        }
        if (lo) b.k0 = 1;
        if (hi) b.k1 = G.kzmax - 2;
        if (b.k1 <= b.k0) return cudaSuccess;
    }
    dim3 gr, bl;
    if (dir < 2) {
        /* r / phi faces marched in runs along their direction: MHD_MARCH_RUN
         * faces per thread where that still gives every SM several blocks,
         * shorter runs on small grids */
        const int nf = dir == 0 ? b.i1 - b.i0 : b.j1 - b.j0;
        const long long lines = (long long)(b.k1 - b.k0) * (dir == 0 ? b.j1 - b.j0 : b.i1 - b.i0);
        const long long want = 4LL * 128 * sm_count();
        const int mr = reflayout || lines * ((nf + MHD_MARCH_RUN - 1) / MHD_MARCH_RUN) >= want ? MHD_MARCH_RUN
                       : lines * ((nf + 3) / 4) >= want ? 4 : 1;
        grid3(b.k1 - b.k0, dir == 0 ? b.j1 - b.j0 : b.i1 - b.i0, (nf + mr - 1) / mr, gr, bl);
#define MHD_MARCH_CASE(D, MR, RL) march_flux_kernel<T, D, MR, RL><<<gr, bl, 0, st>>>(G, V, Vinit, sc, F, b)
        if (reflayout) {
            if (dir == 0) MHD_MARCH_CASE(0, MHD_MARCH_RUN, true); else MHD_MARCH_CASE(1, MHD_MARCH_RUN, true);
        } else if (mr == MHD_MARCH_RUN) {
            if (dir == 0) MHD_MARCH_CASE(0, MHD_MARCH_RUN, false); else MHD_MARCH_CASE(1, MHD_MARCH_RUN, false);
        } else if (mr == 4) {
            if (dir == 0) MHD_MARCH_CASE(0, 4, false); else MHD_MARCH_CASE(1, 4, false);
        } else {
            if (dir == 0) MHD_MARCH_CASE(0, 1, false); else MHD_MARCH_CASE(1, 1, false);
        }
#undef MHD_MARCH_CASE
        return cudaGetLastError();
    }
    /* interior z faces: one warp per (i,j) row, four rows per block */
    const long long nrow = (long long)(b.i1 - b.i0) * (b.j1 - b.j0);
    if (reflayout) zwalk_flux_kernel<T, true><<<nblocks(nrow, 4), 128, 0, st>>>(G, V, sc, F, b);
    else zwalk_flux_kernel<T, false><<<nblocks(nrow, 4), 128, 0, st>>>(G, V, sc, F, b);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_states_t(int dir, const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *Vl,
                            T *Vr, Box b, cudaStream_t st)
{
    if (b.i1 <= b.i0 || b.j1 <= b.j0 || b.k1 <= b.k0) return cudaSuccess;
    dim3 gr, bl;
    grid3(b.k1 - b.k0, b.j1 - b.j0, b.i1 - b.i0, gr, bl);
    if (dir == 0) states_kernel<T, 0><<<gr, bl, 0, st>>>(G, V, Vinit, sc, Vl, Vr, b);
    else if (dir == 1) states_kernel<T, 1><<<gr, bl, 0, st>>>(G, V, Vinit, sc, Vl, Vr, b);
    else states_kernel<T, 2><<<gr, bl, 0, st>>>(G, V, Vinit, sc, Vl, Vr, b);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_update_t(const Geom &G, const StageArgs<T> &a, cudaStream_t st)
{
    const int i1 = a.iend > 0 ? a.iend : G.ixmax - 1;
    if (a.ibeg < 1 || i1 > G.ixmax - 1) return cudaErrorInvalidValue;
    if (i1 <= a.ibeg) return cudaSuccess;
    dim3 gr, bl;
    grid3(G.kzmax - 2, G.jymax - 2, i1 - a.ibeg, gr, bl);
    update_kernel<T><<<gr, bl, 0, st>>>(G, a);
    return cudaGetLastError();
}

/* the TMA-staged update over the tiles that cover the interior planes */
template <typename T>
cudaError_t launch_update_tma_t(const Geom &G, const StageArgs<T> &a, const UpdMaps &maps, int vpar, int *err,
                                cudaStream_t st)
{
    if constexpr (sizeof(T) != 4) {
        return cudaErrorNotSupported;
    } else {
        const long long si = (long long)G.jymax * G.kzmax;
        const long long qbeg = si & ~3LL, qend = (long long)(G.ixmax - 1) * si;
        const long long nt = (qend - qbeg + MHD_UPD_TILE - 1) / MHD_UPD_TILE;
        update_tma_kernel<T><<<(unsigned)nt, MHD_UPD_TILE, 0, st>>>(G, a, maps, vpar, qbeg, err, 1 << 20);
        return cudaGetLastError();
    }
}

/* fused stage launcher: tile 32 (k) x tj (j) cells, runs of seg planes in i */
template <typename T, int TJ>
static cudaError_t stage_attr_t()
{
    constexpr int MINB = sizeof(T) == 4 ? 4 : 2;
    return cudaFuncSetAttribute(stage_kernel<T, TJ, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(StageSmem<T, TJ>));
}

template <typename T>
cudaError_t prepare_stage_t()
{
    return stage_attr_t<T, 7>();
}

template <typename T>
cudaError_t launch_stage_t(const Geom &G, const StageArgs<T> &a, int tj, int seg, cudaStream_t st)
{
    if (seg < 1) seg = 1;
    const int ni = G.ixmax - 2, nj = G.jymax - 2, nk = G.kzmax - 2;
    constexpr int MINB = sizeof(T) == 4 ? 4 : 2;
    dim3 gr((nk + 31) / 32, 0, (ni + seg - 1) / seg);
    if (tj == 7) {
        gr.y = (nj + 6) / 7;
        stage_kernel<T, 7, MINB><<<gr, dim3(32, 8), sizeof(StageSmem<T, 7>), st>>>(G, a, seg);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

/* z fluxes + update launcher: 4 warps of 8 rows per block */
template <typename T>
cudaError_t launch_zupdate_t(const Geom &G, const StageArgs<T> &a, cudaStream_t st)
{
    constexpr int ROWS = 8;
    const long long nrow = (long long)(G.ixmax - 2) * (G.jymax - 2);
    const long long nwarp = (nrow + ROWS - 1) / ROWS;
    zupdate_kernel<T, ROWS><<<(unsigned)((nwarp + 3) / 4), 128, 0, st>>>(G, a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ghost_t(const Geom &G, const StageArgs<T> &a, cudaStream_t st)
{
    const long long ng = ghost_count(G, a.zghost);
    ghost_kernel<T><<<nblocks(ng, 128), 128, 0, st>>>(G, a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_setdt_t(const Geom &G, const T *V, MaxLoc *part, int nblk, cudaStream_t st)
{
    setdt_kernel<T><<<nblk, 256, 0, st>>>(G, V, part);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_source_t(const Geom &G, const T *V, const StepScalars *sc, const double *trig,
                            const float *trigf, double *S, cudaStream_t st)
{
    source_kernel<T><<<nblocks(G.nc, 128), 128, 0, st>>>(G, V, sc, trig, trigf, S);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cvt_t(const double *src, T *dst, long long n, cudaStream_t st)
{
    cvt_from_f64<T><<<1024, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_derive_v_t(const Geom &G, const T *U, T *V, cudaStream_t st)
{
    derive_v_kernel<T><<<(unsigned)(4 * sm_count()), 256, 0, st>>>(G, U, V);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cvt_back_t(const T *src, double *dst, long long n, cudaStream_t st)
{
    cvt_to_f64<T><<<1024, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

} /* namespace mhd */

/* explicit overloads for one T, expanded by the instantiating .cu file */
#define MHD_DEFINE_LAUNCHERS(T)                                                                              \
    namespace mhd {                                                                                          \
    cudaError_t launch_flux(int dir, const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F, \
                            Box b, bool reflayout, cudaStream_t st)                                          \
    {                                                                                                        \
        return launch_flux_t<T>(dir, G, V, Vinit, sc, F, b, reflayout, st);                                  \
    }                                                                                                        \
    cudaError_t launch_flux_zinterior(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc,      \
                                      T *F, Box b, cudaStream_t st)                                          \
    {                                                                                                        \
        return launch_flux_t<T>(2, G, V, Vinit, sc, F, b, false, st, false);                                 \
    }                                                                                                        \
    cudaError_t launch_zedge(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F, Box b,  \
                             cudaStream_t st)                                                                \
    {                                                                                                        \
        return launch_zedge_t<T>(G, V, Vinit, sc, F, b, false, st);                                          \
    }                                                                                                        \
    cudaError_t launch_flux_zwalk(const Geom &G, const T *V, const T *Vinit, const StepScalars *sc, T *F,    \
                                  T *Zs, cudaStream_t st)                                                    \
    {                                                                                                        \
        return launch_flux_zwalk_t<T>(G, V, Vinit, sc, F, Zs, st);                                           \
    }                                                                                                        \
    cudaError_t launch_flux_zlast(const Geom &G, const T *Vinit, const StepScalars *sc, T *H, T *Hb,        \
                                  const T *Zs, int Hfull, cudaStream_t st)                                   \
    {                                                                                                        \
        return launch_flux_zlast_t<T>(G, Vinit, sc, H, Hb, Zs, Hfull, st);                                   \
    }                                                                                                        \
    cudaError_t launch_states(int dir, const Geom &G, const T *V, const T *Vinit, const StepScalars *sc,     \
                              T *Vl, T *Vr, Box b, cudaStream_t st)                                          \
    {                                                                                                        \
        return launch_states_t<T>(dir, G, V, Vinit, sc, Vl, Vr, b, st);                                      \
    }                                                                                                        \
    cudaError_t launch_update(const Geom &G, const StageArgs<T> &a, cudaStream_t st)                          \
    {                                                                                                        \
        return launch_update_t<T>(G, a, st);                                                                 \
    }                                                                                                        \
    cudaError_t launch_update_tma(const Geom &G, const StageArgs<T> &a, const UpdMaps &maps, int vpar,      \
                                  int *err, cudaStream_t st)                                                 \
    {                                                                                                        \
        return launch_update_tma_t<T>(G, a, maps, vpar, err, st);                                            \
    }                                                                                                        \
    cudaError_t launch_ghost(const Geom &G, const StageArgs<T> &a, cudaStream_t st)                           \
    {                                                                                                        \
        return launch_ghost_t<T>(G, a, st);                                                                  \
    }                                                                                                        \
    cudaError_t launch_stage(const Geom &G, const StageArgs<T> &a, int tj, int seg, cudaStream_t st)         \
    {                                                                                                        \
        return launch_stage_t<T>(G, a, tj, seg, st);                                                         \
    }                                                                                                        \
    cudaError_t launch_zupdate(const Geom &G, const StageArgs<T> &a, cudaStream_t st)                       \
    {                                                                                                        \
        return launch_zupdate_t<T>(G, a, st);                                                                \
    }                                                                                                        \
    cudaError_t prepare_stage(T *)                                                                           \
    {                                                                                                        \
        return prepare_stage_t<T>();                                                                         \
    }                                                                                                        \
    cudaError_t launch_setdt(const Geom &G, const T *V, MaxLoc *part, int nblk, cudaStream_t st)            \
    {                                                                                                        \
        return launch_setdt_t<T>(G, V, part, nblk, st);                                                      \
    }                                                                                                        \
    cudaError_t launch_source(const Geom &G, const T *V, const StepScalars *sc, const double *trig,          \
                              const float *trigf, double *S, cudaStream_t st)                                \
    {                                                                                                        \
        return launch_source_t<T>(G, V, sc, trig, trigf, S, st);                                             \
    }                                                                                                        \
    cudaError_t launch_cvt(const double *src, T *dst, long long n, cudaStream_t st)                          \
    {                                                                                                        \
        return launch_cvt_t<T>(src, dst, n, st);                                                             \
    }                                                                                                        \
    cudaError_t launch_cvt_back(const T *src, double *dst, long long n, cudaStream_t st)                     \
    {                                                                                                        \
        return launch_cvt_back_t<T>(src, dst, n, st);                                                        \
    }                                                                                                        \
    cudaError_t launch_derive_v(const Geom &G, const T *U, T *V, cudaStream_t st)                           \
    {                                                                                                        \
        return launch_derive_v_t<T>(G, U, V, st);                                                            \
    }                                                                                                        \
    }

#endif
