/* The call service's doorbell protocol (fgk.h, fgk_serve_words), shared by
 * the compiled kernels' service (fgk_static.cuh) and the generic one
 * (fgk_resident.cu). A service is one CTA: thread 0 waits for the next
 * request with serve_next, the CTA runs it, and thread 0 answers with
 * serve_reply after a barrier. */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"

namespace fgk {

__device__ __forceinline__ uint64_t sv_ld_acquire(const volatile uint64_t *p)
{
	uint64_t v;
	asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ uint64_t sv_ld_relaxed(const volatile void *p)
{
	uint64_t v;
	asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ void sv_st_release(volatile uint64_t *p, uint64_t v)
{
	asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void sv_st_relaxed(volatile uint64_t *p, uint64_t v)
{
	asm volatile("st.relaxed.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

/* the request being served, in shared memory */
struct ServeSlot {
	int      op; /* < 0: leave */
	uint64_t seq;
	uint64_t in, out, kern;
};

/* Thread 0: waits for a doorbell value other than `seen`, at most
 * idle_polls polls in a row. With nothing new it writes 0 to `state`,
 * fences, and reads the doorbell once more (the host stores the doorbell
 * and fences before it reads `state`, so one of the two sees the other):
 * unchanged, the slot says leave; changed, `state` is restored and the
 * request taken. A request with op < 0 also means leave. */
__device__ __forceinline__ void serve_next(const fgk_serve_words &w, uint64_t &seen, uint64_t id,
                                           uint32_t idle_polls, ServeSlot &slot)
{
	uint64_t b = sv_ld_acquire(w.bell);
	for (uint32_t polls = 1; b == seen; polls++) {
		if (polls >= idle_polls) {
			sv_st_release(w.state, 0);
			asm volatile("fence.sc.sys;" ::: "memory");
			b = sv_ld_acquire(w.bell);
			if (b != seen)
				sv_st_relaxed(w.state, id);
			break;
		}
		b = sv_ld_acquire(w.bell);
	}
	slot.op = -1;
	if (b != seen) {
		slot.op = (int)(int32_t)(uint32_t)sv_ld_relaxed(&w.req->op);
		slot.in = sv_ld_relaxed(&w.req->in);
		slot.out = sv_ld_relaxed(&w.req->out);
		slot.kern = sv_ld_relaxed(&w.req->kern);
		slot.seq = b;
		seen = b;
	}
}

/* Thread 0, after a barrier behind the request's stores: one system-scope
 * release of its sequence number (cumulative over the CTA's stores). */
__device__ __forceinline__ void serve_reply(const fgk_serve_words &w, const ServeSlot &slot)
{
	sv_st_release(w.reply, slot.seq);
}

} /* namespace fgk */
