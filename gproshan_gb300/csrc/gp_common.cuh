// Device helpers shared by the kernels: grid barrier with a bounded wait,
// block scans, and the ordered global loads/stores they need.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gp_internal.h"

namespace gp {

// Spin limit of a barrier wait: 2^22 polls with ~128 ns sleeps, about 1-3 s.
// A correct launch never comes near it: the longest wait is one sweep of one
// window (well under a millisecond at the largest sizes).
constexpr uint32_t SPIN_LIMIT = 1u << 22;

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p)
{
	uint32_t v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p)
{
	unsigned long long v;
	asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v)
{
	asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v)
{
	asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t *p, uint32_t v)
{
	uint32_t old;
	asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
	return old;
}

__device__ __forceinline__ unsigned long long atom_add_acquire(unsigned long long *p, unsigned long long v)
{
	unsigned long long old;
	asm volatile("atom.acquire.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
	return old;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p)
{
	uint32_t v;
	asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p)
{
	unsigned long long v;
	asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v)
{
	asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v)
{
	asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}


// Exclusive scan of one value per thread over a block of NT threads.
// *total (shared) receives the block sum.  Every thread must call it.
template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t *total)
{
	static_assert(NT % 32 == 0 && NT <= 1024, "block size");
	__shared__ uint32_t warp_sum[NT / 32];
	__shared__ uint32_t s_total;
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	uint32_t incl = x;
#pragma unroll
	for(int o = 1; o < 32; o <<= 1)
	{
		const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= o) incl += y;
	}
	__syncthreads();
	if(lane == 31) warp_sum[wid] = incl;
	__syncthreads();
	if(wid == 0)
	{
		uint32_t w = lane < NT / 32 ? warp_sum[lane] : 0;
		uint32_t wi = w;
#pragma unroll
		for(int o = 1; o < 32; o <<= 1)
		{
			const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
			if(lane >= o) wi += y;
		}
		if(lane < NT / 32) warp_sum[lane] = wi - w;
		if(lane == NT / 32 - 1) s_total = wi;
	}
	__syncthreads();
	const uint32_t r = incl - x + warp_sum[wid];
	if(total) *total = s_total;
	return r;
}

// Load of a value another CTA of the same persistent launch may have written
// since this CTA last looked (at L2, never from this SM's non-coherent L1).
template <class T>
__device__ __forceinline__ T ldcg(const T *p)
{
	return __ldcg(p);
}

// Index of the last element of sorted `a[0..n)` that is <= key (a[0] <= key).
// CG: `a` may change between grid barriers (coherent loads).
template <bool CG = false>
__device__ __forceinline__ uint32_t upper_index(const uint32_t *a, uint32_t n, uint32_t key)
{
	uint32_t lo = 0, hi = n;  // answer in [lo, hi)
	while(hi - lo > 1)
	{
		const uint32_t mid = (lo + hi) >> 1;
		if((CG ? __ldcg(a + mid) : a[mid]) <= key) lo = mid;
		else hi = mid;
	}
	return lo;
}


} // namespace gp
