// Per-level steps of the toplesets BFS shared by the one-CTA BFS
// (gp_toplesets.cu) and the toplesets built inside the lockstep sweep launch
// (gp_ptp.cu).  See gp_toplesets.cu for the keys and the reference order they
// reproduce (che::compute_toplesets, src/che.cpp:546-593).
#pragma once

#include "gp_common.cuh"

namespace gp {

namespace {

__device__ __forceinline__ uint32_t slot_of(const uint4 &a, const uint4 &b, uint32_t q)
{
	const uint32_t x = q == 0 ? a.x : q == 1 ? a.y : q == 2 ? a.z : q == 3 ? a.w
	                 : q == 4 ? b.x : q == 5 ? b.y : q == 6 ? b.z : b.w;
	return q == 0 && x != FAN8_EMPTY ? x & FAN_MASK : x;
}

// discover: key[u] = min over the frontier of (position << 20 | link slot) + 1.
// No visited test is needed: a vertex met at an earlier level already holds a
// smaller key (its discoverer sat at an earlier position), and the sources
// hold key 0 (set when seeded), so the min leaves them unchanged; a key match
// at emit time therefore means "unvisited and first met here".
// The keys are read first and the atomic is issued only where the key read is
// larger than ours (keys only decrease, so a smaller one stays smaller): on a
// mesh about two thirds of a frontier vertex's links lead back to visited
// vertices, and a level's atomics, all issued by one SM, dominated its time.
// Returns the slots that were not already smaller (the only slots this
// position can own); overflow rows return every slot.
__device__ __forceinline__ uint32_t discover(const FieldDev &F, uint32_t p, uint32_t v, const uint4 &ra, const uint4 &rb)
{
	if(rb.w == FAN8_OVERFLOW)
	{
		const uint32_t o0 = __ldg(F.m.fan_off + v) & FAN_MASK, o1 = __ldg(F.m.fan_off + v + 1) & FAN_MASK;
		for(uint32_t e = o0; e < o1; e++)
			atomicMin(F.key + __ldg(F.m.fan + e), (((unsigned long long) p << 20) | (e - o0)) + 1);
		return 0xFFu;
	}
	unsigned long long k[8];
#pragma unroll
	for(uint32_t q = 0; q < 8; q++)
	{
		const uint32_t u = slot_of(ra, rb, q);
		k[q] = u != FAN8_EMPTY ? ldcg(F.key + u) : 0ull;
	}
	uint32_t cand = 0;
#pragma unroll
	for(uint32_t q = 0; q < 8; q++)
	{
		const unsigned long long mine = (((unsigned long long) p << 20) | q) + 1;
		if(k[q] > mine)
		{
			atomicMin(F.key + slot_of(ra, rb, q), mine);
			cand |= 1u << q;
		}
	}
	return cand;
}

// discover for the one-CTA BFS (bfs_kernel): the same keys, but the visited
// test reads ring[] through L1 instead of the keys through L2.  Only this CTA
// writes the field's rings while its BFS runs (at emit time, ordered before
// the next level by the CTA barrier), and a store from an SM updates that
// SM's L1, so the cached ring of a vertex is current; many of a level's ring
// loads hit lines the previous levels brought in.  A vertex met at this level
// by a frontier position before ours may still get our atomic (its key is
// not read first); the min keeps its key.  The rows of the vertices found are
// prefetched into L1 for the next level, when they are the frontier.
__device__ __forceinline__ uint32_t discover_local(const FieldDev &F, uint32_t p, uint32_t v, const uint4 &ra,
                                                   const uint4 &rb)
{
	if(rb.w == FAN8_OVERFLOW) return discover(F, p, v, ra, rb);
	uint32_t r[8];
#pragma unroll
	for(uint32_t q = 0; q < 8; q++)
	{
		const uint32_t u = slot_of(ra, rb, q);
		r[q] = u != FAN8_EMPTY ? __ldca(F.ring + u) : 0u;
	}
	uint32_t cand = 0;
#pragma unroll
	for(uint32_t q = 0; q < 8; q++)
		if(r[q] == NIL)
		{
			const uint32_t u = slot_of(ra, rb, q);
			atomicMin(F.key + u, (((unsigned long long) p << 20) | q) + 1);
			asm volatile("prefetch.global.L1 [%0];" ::"l"(F.m.fan8 + 2 * (size_t) u));
			cand |= 1u << q;
		}
	return cand;
}

// The vertices owned by frontier position p (key match), as a slot mask;
// overflow rows report their count and are re-walked at emit time.
__device__ __forceinline__ uint32_t owned(const FieldDev &F, uint32_t p, uint32_t v, const uint4 &ra, const uint4 &rb,
                                          uint32_t &count, uint32_t cand = 0xFFu)
{
	uint32_t mask = 0;
	count = 0;
	if(rb.w == FAN8_OVERFLOW)
	{
		const uint32_t o0 = __ldg(F.m.fan_off + v) & FAN_MASK, o1 = __ldg(F.m.fan_off + v + 1) & FAN_MASK;
		for(uint32_t e = o0; e < o1; e++)
			count += ldcg(F.key + __ldg(F.m.fan + e)) == ((((unsigned long long) p << 20) | (e - o0)) + 1);
		return 0;
	}
#pragma unroll
	for(uint32_t q = 0; q < 8; q++)
	{
		const uint32_t u = slot_of(ra, rb, q);
		if((cand >> q & 1u) && u != FAN8_EMPTY && ldcg(F.key + u) == (((unsigned long long) p << 20) | q) + 1)
			mask |= 1u << q;
	}
	count = __popc(mask);
	return mask;
}

} // namespace

} // namespace gp
