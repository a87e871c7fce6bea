/*
 * mhd_fp32.cu -- the precision form's kernels: FP32 state and fluxes with the
 * FP64 repairs written into mhd_dev.cuh (pressure recovery, inner-radius
 * sources, cooling, CFL reduction).
 */
#include "mhd_pair.cuh"

MHD_DEFINE_LAUNCHERS(float)
MHD_DEFINE_PAIR_LAUNCHERS
