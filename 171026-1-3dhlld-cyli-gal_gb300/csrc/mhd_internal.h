/*
 * mhd_internal.h -- declarations shared by the host (.c) and device (.cu)
 * translation units of libmhdgpu.so.  Not part of the public C-ABI.
 */
#ifndef MHD_INTERNAL_H
#define MHD_INTERNAL_H

#include "mhd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* constant.h:62-79 */
#define MHD_GM (5.0 / 3.0)
#define MHD_GM1 (2.0 / 3.0)
#define MHD_ONEOGM1 1.5
#define MHD_ONEOCR (1.0 / 0.18)
#define MHD_ONEO3 (1.0 / 3.0)

#ifdef __cplusplus
}
#endif
#endif
