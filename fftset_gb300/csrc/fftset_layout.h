/* Kernel-buffer layout of the reference (see fftset_layout.c). Internal. */
#ifndef FFTSET_LAYOUT_H
#define FFTSET_LAYOUT_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#define FSL_MAX_CHAIN 64
unsigned fsl_reference_chain(unsigned length, unsigned w, unsigned *chain);
unsigned fsl_lane_width(int freq_offset_real, unsigned L, unsigned simd_width);
/* re_off[bin] = float offset of the real part of bin; imag at + *lanes */
int fsl_kernel_offsets(int freq_offset_real, unsigned L, unsigned simd_width, int32_t *re_off, unsigned *lanes);
#ifdef __cplusplus
}
#endif
#endif
