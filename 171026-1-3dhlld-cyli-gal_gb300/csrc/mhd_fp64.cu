/*
 * mhd_fp64.cu -- the plain FP64 form's kernels.  Compiled with --fmad=false
 * and IEEE division/square root so each expression rounds as the reference C
 * does (the reference is built without contraction as well).
 */
#include "mhd_kernels.cuh"

MHD_DEFINE_LAUNCHERS(double)
