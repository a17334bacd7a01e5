/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * Minimal stand-in for the SIMD layer of the external "cop" library, used
 * only to compile the unmodified fftset sources here as a checker. Lanes are
 * GCC vector extensions; every operation is lane-wise unless stated.
 *
 * ORACLE_VW (1, 4 or 8) selects which vector widths exist, mirroring the
 * V4F_EXISTS / V8F_EXISTS switches fftset tests (src/fftset_vec.c:877,887;
 * src/fftset_mod_freqoffsetreal.c:32,1014-1015; src/fftset_mod_cplx.c:32,322).
 * V4F_EXISTS is left undefined (not 0) for width 1 because
 * src/fftset_mod_freqoffsetreal.c:32 tests it with #ifdef.
 *
 * Macro semantics, each inferred from its use in fftset:
 *   VW_LD2(a,b,p)       a = p[0..W), b = p[W..2W)            (split re/im block)
 *   VW_ST2(p,a,b)       inverse of LD2
 *   VW_ST2INT(p,a,b)    p[2k] = a[k], p[2k+1] = b[k]           (interleave re/im)
 *   VW_LD2DINT(a,b,p)   inverse of ST2INT
 *   VW_ST2X2INT / LD2X2DINT  two ST2INT / LD2DINT at p0 then p1
 *   VW_INTERLEAVE(lo,hi,a,b) lo = a0 b0 a1 b1 ..., hi = second half
 *   VW_DEINTERLEAVE(e,o,lo,hi) inverse of INTERLEAVE
 *   V4F_TRANSPOSE_INPLACE(a,b,c,d)  4x4 transpose of the four rows
 * The forward post-pass of src/fftset_mod_freqoffsetreal.c:520-531 and
 * :832-843 pins INTERLEAVE; the reference's own prime-impulse test program
 * passes at every width when built against this file. */
#ifndef ORACLE_COP_VEC_H
#define ORACLE_COP_VEC_H

#include <string.h>

#ifndef ORACLE_VW
#define ORACLE_VW 4
#endif

#define COP_ATTR_ALWAYSINLINE inline __attribute__((always_inline))
#define VEC_ALIGN_BEST        __attribute__((aligned(64)))

typedef float v1f;
#define v1f_ld(p_)          (*(p_))
#define v1f_st(p_, a_)      (*(p_) = (a_))
#define v1f_add(a_, b_)     ((a_) + (b_))
#define v1f_sub(a_, b_)     ((a_) - (b_))
#define v1f_mul(a_, b_)     ((a_) * (b_))
#define v1f_neg(a_)         (-(a_))
#define v1f_broadcast(a_)   (a_)
#define V1F_LD2(a_, b_, p_) do { (a_) = (p_)[0]; (b_) = (p_)[1]; } while (0)
#define V1F_ST2(p_, a_, b_) do { (p_)[0] = (a_); (p_)[1] = (b_); } while (0)

#if ORACLE_VW >= 4
#define V4F_EXISTS 1
typedef float v4f __attribute__((vector_size(16)));
static inline v4f  v4f_ld(const float *p) { v4f r; memcpy(&r, p, sizeof r); return r; }
static inline void v4f_st(float *p, v4f a) { memcpy(p, &a, sizeof a); }
static inline v4f  v4f_broadcast(float x) { v4f r = {x, x, x, x}; return r; }
static inline v4f  v4f_reverse(v4f a) { v4f r = {a[3], a[2], a[1], a[0]}; return r; }
#define v4f_add(a_, b_) ((a_) + (b_))
#define v4f_sub(a_, b_) ((a_) - (b_))
#define v4f_mul(a_, b_) ((a_) * (b_))
#define v4f_neg(a_)     (-(a_))
#define V4F_LD2(a_, b_, p_) do { (a_) = v4f_ld(p_); (b_) = v4f_ld((p_) + 4); } while (0)
#define V4F_ST2(p_, a_, b_) do { v4f_st((p_), (a_)); v4f_st((p_) + 4, (b_)); } while (0)
#define V4F_ST2INT(p_, a_, b_) do { int k_; for (k_ = 0; k_ < 4; k_++) { (p_)[2*k_] = (a_)[k_]; (p_)[2*k_+1] = (b_)[k_]; } } while (0)
#define V4F_LD2DINT(a_, b_, p_) do { int k_; for (k_ = 0; k_ < 4; k_++) { (a_)[k_] = (p_)[2*k_]; (b_)[k_] = (p_)[2*k_+1]; } } while (0)
#define V4F_ST2X2INT(p0_, p1_, a_, b_, c_, d_) do { V4F_ST2INT(p0_, a_, b_); V4F_ST2INT(p1_, c_, d_); } while (0)
#define V4F_LD2X2DINT(a_, b_, c_, d_, p0_, p1_) do { V4F_LD2DINT(a_, b_, p0_); V4F_LD2DINT(c_, d_, p1_); } while (0)
#define V4F_INTERLEAVE(lo_, hi_, a_, b_) do { \
	v4f l_ = {(a_)[0], (b_)[0], (a_)[1], (b_)[1]}; \
	v4f h_ = {(a_)[2], (b_)[2], (a_)[3], (b_)[3]}; \
	(lo_) = l_; (hi_) = h_; } while (0)
#define V4F_DEINTERLEAVE(ev_, od_, lo_, hi_) do { \
	v4f e_ = {(lo_)[0], (lo_)[2], (hi_)[0], (hi_)[2]}; \
	v4f o_ = {(lo_)[1], (lo_)[3], (hi_)[1], (hi_)[3]}; \
	(ev_) = e_; (od_) = o_; } while (0)
#define V4F_TRANSPOSE_INPLACE(a_, b_, c_, d_) do { \
	v4f t0_ = {(a_)[0], (b_)[0], (c_)[0], (d_)[0]}; \
	v4f t1_ = {(a_)[1], (b_)[1], (c_)[1], (d_)[1]}; \
	v4f t2_ = {(a_)[2], (b_)[2], (c_)[2], (d_)[2]}; \
	v4f t3_ = {(a_)[3], (b_)[3], (c_)[3], (d_)[3]}; \
	(a_) = t0_; (b_) = t1_; (c_) = t2_; (d_) = t3_; } while (0)
#endif

#if ORACLE_VW >= 8
#define V8F_EXISTS 1
typedef float v8f __attribute__((vector_size(32)));
static inline v8f  v8f_ld(const float *p) { v8f r; memcpy(&r, p, sizeof r); return r; }
static inline void v8f_st(float *p, v8f a) { memcpy(p, &a, sizeof a); }
static inline v8f  v8f_broadcast(float x) { v8f r = {x, x, x, x, x, x, x, x}; return r; }
static inline v8f  v8f_reverse(v8f a) { v8f r; int k; for (k = 0; k < 8; k++) r[k] = a[7 - k]; return r; }
#define v8f_add(a_, b_) ((a_) + (b_))
#define v8f_sub(a_, b_) ((a_) - (b_))
#define v8f_mul(a_, b_) ((a_) * (b_))
#define v8f_neg(a_)     (-(a_))
#define V8F_LD2(a_, b_, p_) do { (a_) = v8f_ld(p_); (b_) = v8f_ld((p_) + 8); } while (0)
#define V8F_ST2(p_, a_, b_) do { v8f_st((p_), (a_)); v8f_st((p_) + 8, (b_)); } while (0)
#define V8F_ST2INT(p_, a_, b_) do { int k_; for (k_ = 0; k_ < 8; k_++) { (p_)[2*k_] = (a_)[k_]; (p_)[2*k_+1] = (b_)[k_]; } } while (0)
#define V8F_LD2DINT(a_, b_, p_) do { int k_; for (k_ = 0; k_ < 8; k_++) { (a_)[k_] = (p_)[2*k_]; (b_)[k_] = (p_)[2*k_+1]; } } while (0)
#define V8F_ST2X2INT(p0_, p1_, a_, b_, c_, d_) do { V8F_ST2INT(p0_, a_, b_); V8F_ST2INT(p1_, c_, d_); } while (0)
#define V8F_LD2X2DINT(a_, b_, c_, d_, p0_, p1_) do { V8F_LD2DINT(a_, b_, p0_); V8F_LD2DINT(c_, d_, p1_); } while (0)
#define V8F_INTERLEAVE(lo_, hi_, a_, b_) do { int k_; v8f l_, h_; \
	for (k_ = 0; k_ < 4; k_++) { l_[2*k_] = (a_)[k_]; l_[2*k_+1] = (b_)[k_]; h_[2*k_] = (a_)[k_+4]; h_[2*k_+1] = (b_)[k_+4]; } \
	(lo_) = l_; (hi_) = h_; } while (0)
#define V8F_DEINTERLEAVE(ev_, od_, lo_, hi_) do { int k_; v8f e_, o_; \
	for (k_ = 0; k_ < 4; k_++) { e_[k_] = (lo_)[2*k_]; o_[k_] = (lo_)[2*k_+1]; e_[k_+4] = (hi_)[2*k_]; o_[k_+4] = (hi_)[2*k_+1]; } \
	(ev_) = e_; (od_) = o_; } while (0)
#endif

#endif
