/* Allocation wrappers of the host layer.
 *
 * Every host (malloc, calloc) and device (cudaMalloc, cudaHostAlloc)
 * allocation made by fftset_host.c, fftset_ragged.c, fftset_adjoint.c,
 * fftset_ola.c and fftset_tuning.c goes through these functions
 * (fftset_internal.h maps the names). They count the allocations still held
 * and can be told to make one allocation fail, so that tests can check the
 * reference's failure contract without exhausting real memory: fftset_init
 * returns non-zero and fftset_create_fft returns NULL when memory runs out
 * (fftset.h:44-47, :78; src/fftset.c:84, :112-116), with nothing leaked. */
#define FS_ALLOC_IMPL
#include <stdlib.h>

#include <cuda_runtime_api.h>

#include "fftset_internal.h"

static long fs_fail_countdown; /* > 0: the allocation that brings it to 0 fails */
static long fs_live_host, fs_live_dev;

static int fs_inject_failure(void)
{
	long n = __atomic_load_n(&fs_fail_countdown, __ATOMIC_ACQUIRE);
	if (n <= 0)
		return 0;
	return __atomic_sub_fetch(&fs_fail_countdown, 1, __ATOMIC_ACQ_REL) == 0;
}

void *fs_malloc(size_t n)
{
	void *p = fs_inject_failure() ? NULL : malloc(n);
	if (p)
		__atomic_add_fetch(&fs_live_host, 1, __ATOMIC_RELAXED);
	return p;
}

void *fs_calloc(size_t n, size_t m)
{
	void *p = fs_inject_failure() ? NULL : calloc(n, m);
	if (p)
		__atomic_add_fetch(&fs_live_host, 1, __ATOMIC_RELAXED);
	return p;
}

void fs_free(void *p)
{
	if (p) {
		__atomic_sub_fetch(&fs_live_host, 1, __ATOMIC_RELAXED);
		free(p);
	}
}

cudaError_t fs_cuda_malloc(void **p, size_t n)
{
	cudaError_t e;
	if (fs_inject_failure()) {
		*p = NULL;
		return cudaErrorMemoryAllocation;
	}
	e = cudaMalloc(p, n);
	if (e == cudaSuccess)
		__atomic_add_fetch(&fs_live_dev, 1, __ATOMIC_RELAXED);
	return e;
}

cudaError_t fs_cuda_free(void *p)
{
	cudaError_t e;
	if (!p)
		return cudaSuccess;
	e = cudaFree(p);
	if (e == cudaSuccess)
		__atomic_sub_fetch(&fs_live_dev, 1, __ATOMIC_RELAXED);
	return e;
}

cudaError_t fs_cuda_host_alloc(void **p, size_t n, unsigned flags)
{
	cudaError_t e;
	if (fs_inject_failure()) {
		*p = NULL;
		return cudaErrorMemoryAllocation;
	}
	e = cudaHostAlloc(p, n, flags);
	if (e == cudaSuccess)
		__atomic_add_fetch(&fs_live_dev, 1, __ATOMIC_RELAXED);
	return e;
}

cudaError_t fs_cuda_free_host(void *p)
{
	cudaError_t e;
	if (!p)
		return cudaSuccess;
	e = cudaFreeHost(p);
	if (e == cudaSuccess)
		__atomic_sub_fetch(&fs_live_dev, 1, __ATOMIC_RELAXED);
	return e;
}

/* Test hooks (declared in fftset_internal.h, not in the public header). */
long fftset__test_fail_allocation(long nth)
{
	return __atomic_exchange_n(&fs_fail_countdown, nth > 0 ? nth : 0, __ATOMIC_ACQ_REL);
}

void fftset__test_live_allocations(long *host, long *device)
{
	if (host)
		*host = __atomic_load_n(&fs_live_host, __ATOMIC_ACQUIRE);
	if (device)
		*device = __atomic_load_n(&fs_live_dev, __ATOMIC_ACQUIRE);
}
