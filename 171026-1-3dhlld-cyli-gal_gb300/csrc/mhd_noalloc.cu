/*
 * mhd_noalloc.cu -- mhd_setdt_noalloc(): the CFL reduction (the same
 * setdt_kernel as mhd_setdt) for callers that cannot allocate device memory.
 *
 * Some callers may not call cudaMalloc at the moment they need a time step:
 * a host that hands out all device memory from its own pool at start-up and
 * forbids allocation afterwards, a real-time or embedded loop that must not
 * touch the allocator, or code running while another component holds the
 * allocator.  mhd_setdt() keeps its per-block partial maxima in a buffer the
 * context allocated; this variant keeps them in a fixed file-scope device
 * array instead and allocates nothing on the host or the device.
 *
 * The scratch is MHD_NOALLOC_MAX_BLOCKS partial results (16 bytes each) plus
 * one result slot: about 128 KB that every GPU which loads this library holds
 * until the process exits.  Each call shares it and leaves its own contents
 * there; every slot a call reads was written by that call, so nothing needs
 * clearing.  Two calls that overlap on the GPU (different streams or host
 * threads) race on the array and must be serialised by the caller.
 *
 * In host code the array's name is only a host-side stand-in for the device
 * symbol, so its device address is looked up once per device with
 * cudaGetSymbolAddress() -- on the first call made with that device current.
 * That first call should therefore come before any stream capture.
 */
#include <cuda_runtime.h>

#include <string.h>

#include <mutex>

#include "mhd_kernels.cuh"

using namespace mhd;

#define MHD_NOALLOC_CELLS_PER_THREAD 64
#define MHD_NOALLOC_THREADS 256
#define MHD_NOALLOC_MAX_DEVICES 64

/* MHD_NOALLOC_MAX_BLOCKS partials + 1 result slot */
static __device__ __align__(256) MaxLoc g_noalloc_scratch[MHD_NOALLOC_MAX_BLOCKS + 1];

static std::mutex g_noalloc_mutex;
static MaxLoc *g_noalloc_ptr[MHD_NOALLOC_MAX_DEVICES];

/* one block folds the partials with the same tie rule as the host fold of
 * mhd_setdt (larger value, then smaller cell index) */
__global__ void noalloc_fold_kernel(const MaxLoc *__restrict__ part, int n, MaxLoc *out)
{
    __shared__ MaxLoc sm[32];
    MaxLoc best = {0.0, -1};
    for (int b = threadIdx.x; b < n; b += blockDim.x) best = better(best, part[b]);
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
        *out = b;
    }
}

static int scratch_for_current_device(MaxLoc **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return MHD_ERR_CUDA;
    if (dev < 0 || dev >= MHD_NOALLOC_MAX_DEVICES) return MHD_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = NULL;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MHD_ERR_CUDA;
        g_noalloc_ptr[dev] = (MaxLoc *)p;
    }
    *out = g_noalloc_ptr[dev];
    return MHD_OK;
}

extern "C" int mhd_setdt_noalloc(const double *V, const double *minlength, int ix, int jy, int kz, double cfl,
                                 double minminlength, int cooling, void *stream, double *dt, double *ch,
                                 int ijk[3])
{
    if (!V || !minlength || !dt || !ch || ix < 12 || jy < 1 || kz < 1) return MHD_ERR_ARG;
    const long long ncfl = (long long)(ix - 10) * jy * kz;   /* setdt.h:33-35 range */
    const long long per_block = (long long)MHD_NOALLOC_THREADS * MHD_NOALLOC_CELLS_PER_THREAD;
    const long long nblk = (ncfl + per_block - 1) / per_block;
    if (nblk > MHD_NOALLOC_MAX_BLOCKS) return MHD_ERR_ARG;   /* beyond the fixed scratch */

    MaxLoc *scratch = NULL;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;

    Geom G;
    memset((void *)&G, 0, sizeof G);
    G.ixmax = ix + 2;
    G.jymax = jy + 2;
    G.kzmax = kz + 2;
    G.jy = jy;
    G.nc = (long long)G.ixmax * G.jymax * G.kzmax;
    G.minlength = minlength;
    G.cooling = cooling;
    cudaStream_t st = (cudaStream_t)stream;
    setdt_kernel<double><<<(unsigned)nblk, MHD_NOALLOC_THREADS, 0, st>>>(G, V, scratch);
    if (cudaGetLastError() != cudaSuccess) return MHD_ERR_CUDA;
    noalloc_fold_kernel<<<1, 1024, 0, st>>>(scratch, (int)nblk, scratch + MHD_NOALLOC_MAX_BLOCKS);
    if (cudaGetLastError() != cudaSuccess) return MHD_ERR_CUDA;
    MaxLoc best;
    if (cudaMemcpyAsync(&best, scratch + MHD_NOALLOC_MAX_BLOCKS, sizeof best, cudaMemcpyDeviceToHost, st) !=
        cudaSuccess)
        return MHD_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MHD_ERR_CUDA;
    double oneocfldt = best.q >= 0 ? best.v : 0.0;
    *dt = cfl / oneocfldt;            /* setdt.h:84 */
    *ch = minminlength * oneocfldt;   /* setdt.h:89 */
    if (ijk) {
        if (best.q < 0) { ijk[0] = ijk[1] = ijk[2] = -1; }
        else {
            ijk[2] = (int)(best.q % G.kzmax);
            ijk[1] = (int)((best.q / G.kzmax) % G.jymax);
            ijk[0] = (int)(best.q / ((long long)G.kzmax * G.jymax));
        }
    }
    return MHD_OK;
}
