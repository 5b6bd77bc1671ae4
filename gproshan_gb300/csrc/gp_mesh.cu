// Mesh upload kernels: star lists ("fans") built from the compact half-edge
// tables, coordinate conversion, and the device scan used by every layout pass.
//
// A vertex's fan is the sequence of link vertices met by the reference's star
// walk (for_star, include/che.h:10): for each half-edge he of the star, in walk
// order, the vertex VT[next(he)]; when the walk ends on a border
// (OT[prev(he)] == NIL) the last VT[prev(he)] follows.  This is exactly
// che::link (src/che.cpp:102-112), so the BFS reads it as the link, and the
// relaxation reads consecutive pairs as the star triangles (x0 = VT[next(he)],
// x1 = VT[prev(he)], src/geodesics_ptp.cpp:203-205): on a closed fan the last
// pair wraps to the first entry.
#include "gp_common.cuh"

namespace gp {

namespace {

constexpr int SCAN_NT = 256;
constexpr int SCAN_IPT = 4;
constexpr int SCAN_TILE = SCAN_NT * SCAN_IPT;

__global__ void fan_count_kernel(const uint32_t *__restrict__ VT, const uint32_t *__restrict__ OT,
                                 const uint32_t *__restrict__ EVT, uint32_t nv, uint32_t nhe,
                                 uint32_t *__restrict__ cnt, uint32_t *__restrict__ err)
{
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if(v >= nv) return;
	const uint32_t he0 = EVT[v];
	uint32_t c = 0, closed = 0;
	if(he0 != NIL)
	{
		if(he0 >= nhe) { atomicOr(err, DEV_ERR_BOUNDS); cnt[v] = 0; return; }
		uint32_t he = he0, T = 0;
		for(;;)
		{
			T++;
			const uint32_t nx = OT[he_prev(he)];
			if(nx == NIL) break;
			if(nx == he0) { closed = 1; break; }
			if(nx >= nhe || T >= MAX_WALK) { atomicOr(err, nx >= nhe ? DEV_ERR_BOUNDS : DEV_ERR_WALK); T = 0; break; }
			he = nx;
		}
		c = T ? (closed ? T : T + 1) : 0;
	}
	cnt[v] = c | (closed ? FAN_CLOSED : 0u);
}

__global__ void strip_flag_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, uint32_t n)
{
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if(v < n) out[v] = in[v] & FAN_MASK;
}

__global__ void fan_fill_kernel(const uint32_t *__restrict__ VT, const uint32_t *__restrict__ OT,
                                const uint32_t *__restrict__ EVT, uint32_t nv,
                                const uint32_t *__restrict__ flags, uint32_t *__restrict__ off,
                                uint32_t *__restrict__ fan)
{
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if(v >= nv) return;
	const uint32_t f = flags[v];
	const uint32_t n = f & FAN_MASK;
	const uint32_t o = off[v];
	if(n)
	{
		const uint32_t he0 = EVT[v];
		uint32_t he = he0, k = 0;
		for(;;)
		{
			fan[o + k++] = VT[he_next(he)];
			const uint32_t nx = OT[he_prev(he)];
			if(nx == NIL) { fan[o + k++] = VT[he_prev(he)]; break; }
			if(nx == he0 || k >= n) break;
			he = nx;
		}
	}
	off[v] = o | (f & FAN_CLOSED);
}

// Fixed-stride rows of the links (see FAN8_* in gp_internal.h).
__global__ void fan8_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ fan, uint32_t nv,
                            uint4 *__restrict__ rows)
{
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if(v >= nv) return;
	const uint32_t o0f = off[v], o0 = o0f & FAN_MASK, o1 = off[v + 1] & FAN_MASK;
	const uint32_t n = o1 - o0;
	uint32_t r[8];
	for(uint32_t q = 0; q < 8; q++) r[q] = q < n ? fan[o0 + q] : FAN8_EMPTY;
	if(n > 8) r[7] = FAN8_OVERFLOW;
	if(n && (o0f & FAN_CLOSED)) r[0] |= FAN_CLOSED;
	rows[2 * (size_t) v] = make_uint4(r[0], r[1], r[2], r[3]);
	rows[2 * (size_t) v + 1] = make_uint4(r[4], r[5], r[6], r[7]);
}

// Per face: its three edge lengths (each edge counted from both sides, so
// every interior edge twice: the averages are unaffected), whether it is
// obtuse, and for each interior edge the dihedral deviation 1 - n1.n2.
__global__ void mesh_stats_kernel(const uint32_t *__restrict__ VT, const uint32_t *__restrict__ OT,
                                  const float4 *__restrict__ pos, uint32_t nf, double *acc)
{
	double l1 = 0, l2 = 0, g1 = 0, g2 = 0, ne = 0, obt = 0, dih = 0, ni = 0;
	for(uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += gridDim.x * blockDim.x)
	{
		const float4 a = pos[VT[3 * t]], b = pos[VT[3 * t + 1]], c = pos[VT[3 * t + 2]];
		const float3 e0 = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
		const float3 e1 = make_float3(c.x - b.x, c.y - b.y, c.z - b.z);
		const float3 e2 = make_float3(a.x - c.x, a.y - c.y, a.z - c.z);
		const float q[3] = {e0.x * e0.x + e0.y * e0.y + e0.z * e0.z, e1.x * e1.x + e1.y * e1.y + e1.z * e1.z,
		                    e2.x * e2.x + e2.y * e2.y + e2.z * e2.z};
		for(int k = 0; k < 3; k++)
			if(q[k] > 0.f)
			{
				const double l = sqrt((double) q[k]), g = log(l);
				l1 += l;
				l2 += l * l;
				g1 += g;
				g2 += g * g;
				ne += 1;
			}
		const float qm = fmaxf(q[0], fmaxf(q[1], q[2]));
		obt += 2.f * qm > q[0] + q[1] + q[2];  // q_max > q_other1 + q_other2
		float3 n = make_float3(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x);
		const float nn = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
		for(int k = 0; k < 3; k++)
		{
			const uint32_t o = OT[3 * t + k];
			if(o == NIL || o / 3 < t || nn <= 0.f) continue;  // each interior edge once
			const uint32_t u = o / 3;
			const float4 A = pos[VT[3 * u]], B = pos[VT[3 * u + 1]], C = pos[VT[3 * u + 2]];
			const float3 f0 = make_float3(B.x - A.x, B.y - A.y, B.z - A.z);
			const float3 f1 = make_float3(C.x - B.x, C.y - B.y, C.z - B.z);
			const float3 m = make_float3(f0.y * f1.z - f0.z * f1.y, f0.z * f1.x - f0.x * f1.z, f0.x * f1.y - f0.y * f1.x);
			const float mm = sqrtf(m.x * m.x + m.y * m.y + m.z * m.z);
			if(mm <= 0.f) continue;
			dih += 1.0 - (double) ((n.x * m.x + n.y * m.y + n.z * m.z) / (nn * mm));
			ni += 1;
		}
	}
	double v[8] = {l1, l2, g1, g2, ne, obt, dih, ni};
	for(int k = 0; k < 8; k++)
	{
		double x = v[k];
		for(int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
		if((threadIdx.x & 31) == 0) atomicAdd(acc + k, x);
	}
}

__global__ void max_kernel(const uint32_t *__restrict__ in, size_t n, uint32_t *out)
{
	uint32_t m = 0;
	for(size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x)
		m = max(m, in[i] & FAN_MASK);
	for(int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
	if((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void pos_kernel(const double *__restrict__ xyz, uint32_t nv, float4 *__restrict__ pos,
                           double *__restrict__ posd)
{
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if(v >= nv) return;
	const double x = xyz[3 * (size_t) v], y = xyz[3 * (size_t) v + 1], z = xyz[3 * (size_t) v + 2];
	pos[v] = make_float4((float) x, (float) y, (float) z, 0.f);
	if(posd)
	{
		posd[4 * (size_t) v] = x;
		posd[4 * (size_t) v + 1] = y;
		posd[4 * (size_t) v + 2] = z;
		posd[4 * (size_t) v + 3] = 0.0;
	}
}

// --- scan: per-tile sums, recursive scan of the sums, then per-tile scan ----

__global__ void scan_reduce_kernel(const uint32_t *__restrict__ in, size_t n, uint32_t *__restrict__ sums)
{
	const size_t base = (size_t) blockIdx.x * SCAN_TILE;
	uint32_t s = 0;
#pragma unroll
	for(int k = 0; k < SCAN_IPT; k++)
	{
		const size_t i = base + (size_t) threadIdx.x * SCAN_IPT + k;
		if(i < n) s += in[i];
	}
	for(int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	__shared__ uint32_t ws[SCAN_NT / 32];
	if((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		uint32_t t = 0;
		for(int w = 0; w < SCAN_NT / 32; w++) t += ws[w];
		sums[blockIdx.x] = t;
	}
}

__global__ void scan_tile_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, size_t n,
                                 const uint32_t *__restrict__ tile_off, int write_total)
{
	const size_t base = (size_t) blockIdx.x * SCAN_TILE;
	uint32_t v[SCAN_IPT];
	uint32_t s = 0;
#pragma unroll
	for(int k = 0; k < SCAN_IPT; k++)
	{
		const size_t i = base + (size_t) threadIdx.x * SCAN_IPT + k;
		v[k] = i < n ? in[i] : 0u;
		s += v[k];
	}
	uint32_t tot;
	const uint32_t ex = block_exclusive_scan<SCAN_NT>(s, &tot);
	uint32_t run = ex + (tile_off ? tile_off[blockIdx.x] : 0u);
#pragma unroll
	for(int k = 0; k < SCAN_IPT; k++)
	{
		const size_t i = base + (size_t) threadIdx.x * SCAN_IPT + k;
		if(i < n) out[i] = run;
		run += v[k];
	}
	if(write_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_NT - 1) out[n] = run;
}

// ---------------------------------------------------------------------------
// Half-edge tables on the GPU: che::update_evt_ot_et (src/che.cpp:1295-1362)
// in parallel, with its exact results, non-manifold cases included.
//
// The reference pairs half-edges greedily in half-edge order: an unpaired he
// (a -> b) takes the first still-free t (b -> a) in the order of next(t).  Its
// choices for one undirected edge {a, b} only involve the half-edges lying on
// that edge, so the greedy splits into independent groups: the half-edges are
// grouped by edge in a hash table, each group's smallest member runs the
// greedy on its group (the usual group of one or two is settled at once), and
// each vertex replays the border rule for EVT over its own border half-edges
// in half-edge order.  A group or border list longer than CHE_LOCAL entries
// sets a flag (the host then builds the tables instead).
// ---------------------------------------------------------------------------
constexpr uint32_t CHE_LOCAL = 32;
constexpr unsigned long long CHE_EMPTY = ~0ull;

__device__ __forceinline__ uint32_t che_hash(unsigned long long k, uint32_t mask)
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdull;
	k ^= k >> 33;
	return (uint32_t) k & mask;
}

// EVT (last half-edge of each vertex, +1), the edge groups, per-vertex lists
__global__ void che_group_kernel(const uint32_t *__restrict__ VT, uint32_t nhe, uint32_t nv,
                                 unsigned long long *keys, uint32_t *heads, uint32_t mask, uint32_t *grp,
                                 uint32_t *nextg, uint32_t *evt1, uint32_t *err)
{
	const uint32_t he = blockIdx.x * blockDim.x + threadIdx.x;
	if(he >= nhe) return;
	const uint32_t a = VT[he], b = VT[he_next(he)];
	if(a >= nv || b >= nv)
	{
		atomicOr(err, DEV_ERR_BOUNDS);
		return;
	}
	atomicMax(evt1 + a, he + 1);
	const unsigned long long key = ((unsigned long long) min(a, b) << 32) | max(a, b);
	uint32_t slot = che_hash(key, mask);
	for(uint32_t probe = 0; probe <= mask; probe++)
	{
		const unsigned long long prev = atomicCAS(keys + slot, CHE_EMPTY, key);
		if(prev == CHE_EMPTY || prev == key)
		{
			grp[he] = slot;
			nextg[he] = atomicExch(heads + slot, he);
			return;
		}
		slot = (slot + 1) & mask;
	}
	atomicOr(err, DEV_ERR_BOUNDS);  // table full: cannot happen at 2x load
}

__device__ __forceinline__ void sort_small(uint32_t *x, uint32_t n)
{
	for(uint32_t i = 1; i < n; i++)
	{
		const uint32_t v = x[i];
		uint32_t j = i;
		for(; j && x[j - 1] > v; j--) x[j] = x[j - 1];
		x[j] = v;
	}
}

__global__ void che_pair_kernel(const uint32_t *__restrict__ VT, uint32_t nhe, const uint32_t *heads,
                                const uint32_t *grp, const uint32_t *nextg, uint32_t *OT, uint32_t *err)
{
	const uint32_t he = blockIdx.x * blockDim.x + threadIdx.x;
	if(he >= nhe) return;
	// the group's smallest member does the group's work
	uint32_t m[CHE_LOCAL], n = 0, lo = he;
	bool over = false;
	for(uint32_t x = heads[grp[he]]; x != NIL; x = nextg[x])
	{
		lo = min(lo, x);
		if(n < CHE_LOCAL) m[n++] = x;
		else over = true;
	}
	if(lo != he) return;
	if(over)
	{
		atomicOr(err, 8u);
		return;
	}
	sort_small(m, n);
	for(uint32_t k = 0; k < n; k++) OT[m[k]] = NIL;
	for(uint32_t k = 0; k < n; k++)
	{
		const uint32_t x = m[k];
		if(OT[x] != NIL) continue;
		const uint32_t a = VT[x], b = VT[he_next(x)];
		// candidates t (b -> a) of the group, in the order of next(t)
		uint32_t cand[CHE_LOCAL], nc = 0;
		for(uint32_t q = 0; q < n; q++)
		{
			const uint32_t t = m[q];
			if(VT[t] == b && VT[he_next(t)] == a) cand[nc++] = he_next(t);
		}
		sort_small(cand, nc);
		for(uint32_t q = 0; q < nc; q++)
		{
			const uint32_t t = he_prev(cand[q]);
			if(OT[x] == NIL && OT[t] == NIL)
			{
				OT[x] = t;
				OT[t] = x;
			}
		}
	}
}

// border half-edges listed per vertex
__global__ void che_border_kernel(const uint32_t *__restrict__ VT, const uint32_t *__restrict__ OT, uint32_t nhe,
                                  uint32_t *bhead, uint32_t *bnext)
{
	const uint32_t he = blockIdx.x * blockDim.x + threadIdx.x;
	if(he >= nhe || OT[he] != NIL) return;
	bnext[he] = atomicExch(bhead + VT[he], he);
}

// EVT: the last half-edge of the vertex, then the border rule replayed over
// the vertex's border half-edges in order; flags[1] = 1 if non-manifold
__global__ void che_evt_kernel(const uint32_t *__restrict__ OT, uint32_t nv, const uint32_t *evt1,
                               const uint32_t *bhead, const uint32_t *bnext, uint32_t *EVT, uint32_t *err,
                               uint32_t *nonmanifold)
{
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if(v >= nv) return;
	uint32_t e = evt1[v] - 1u;  // NIL when the vertex has no half-edge
	uint32_t b[CHE_LOCAL], n = 0;
	for(uint32_t x = bhead[v]; x != NIL; x = bnext[x])
	{
		if(n == CHE_LOCAL)
		{
			atomicOr(err, 8u);
			return;
		}
		b[n++] = x;
	}
	sort_small(b, n);
	for(uint32_t k = 0; k < n; k++)
	{
		if(e == NIL) continue;
		if(OT[e] == NIL && e != b[k])
		{
			e = NIL;
			atomicExch(nonmanifold, 1u);
		}
		else e = b[k];
	}
	EVT[v] = e;
}

} // namespace

size_t che_build_scratch_bytes(uint32_t nv, uint32_t nhe)
{
	uint32_t T = 1;
	while(T < 2 * std::max(nhe, 1u)) T <<= 1;
	return 8ull * T + 4ull * T + 4ull * nhe * 3 + 4ull * nv * 2 + 4096;
}

// VT (device) -> OT, EVT (device).  flags: 4 words, [0] error bits (8: a
// group or border list too long for the GPU build), [1] non-manifold.
cudaError_t launch_che_build(const uint32_t *VT, uint32_t nv, uint32_t nhe, uint32_t *OT, uint32_t *EVT,
                             void *scratch, uint32_t *flags, cudaStream_t s)
{
	uint32_t T = 1;
	while(T < 2 * std::max(nhe, 1u)) T <<= 1;
	char *p = static_cast<char *>(scratch);
	unsigned long long *keys = reinterpret_cast<unsigned long long *>(p);
	uint32_t *heads = reinterpret_cast<uint32_t *>(keys + T);
	uint32_t *grp = heads + T, *nextg = grp + nhe, *bnext = nextg + nhe;
	uint32_t *evt1 = bnext + nhe, *bhead = evt1 + nv;
	cudaError_t e = cudaMemsetAsync(keys, 0xFF, 8ull * T, s);
	if(e == cudaSuccess) e = cudaMemsetAsync(heads, 0xFF, 4ull * T, s);
	if(e == cudaSuccess) e = cudaMemsetAsync(evt1, 0, 4ull * nv, s);
	if(e == cudaSuccess) e = cudaMemsetAsync(bhead, 0xFF, 4ull * nv, s);
	if(e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 16, s);
	if(e != cudaSuccess) return e;
	const unsigned gh = (nhe + 255) / 256, gv = (nv + 255) / 256;
	if(nhe)
	{
		che_group_kernel<<<gh, 256, 0, s>>>(VT, nhe, nv, keys, heads, T - 1, grp, nextg, evt1, flags);
		che_pair_kernel<<<gh, 256, 0, s>>>(VT, nhe, heads, grp, nextg, OT, flags);
		che_border_kernel<<<gh, 256, 0, s>>>(VT, OT, nhe, bhead, bnext);
	}
	if(nv) che_evt_kernel<<<gv, 256, 0, s>>>(OT, nv, evt1, bhead, bnext, EVT, flags, flags + 1);
	return cudaGetLastError();
}

size_t scan_tmp_words(size_t n)
{
	size_t words = 0;
	while(n > (size_t) SCAN_TILE)
	{
		const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
		words += nb + 1;
		n = nb;
	}
	return words + 1;
}

cudaError_t launch_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *tmp, cudaStream_t s)
{
	if(n == 0)
		return cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
	if(n <= (size_t) SCAN_TILE)
	{
		scan_tile_kernel<<<1, SCAN_NT, 0, s>>>(in, out, n, nullptr, 1);
		return cudaGetLastError();
	}
	const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
	uint32_t *sums = tmp;          // nb + 1 entries (scanned in place)
	uint32_t *rest = tmp + nb + 1;
	scan_reduce_kernel<<<(unsigned) nb, SCAN_NT, 0, s>>>(in, n, sums);
	cudaError_t e = launch_scan_u32(sums, sums, nb, rest, s);
	if(e != cudaSuccess) return e;
	scan_tile_kernel<<<(unsigned) nb, SCAN_NT, 0, s>>>(in, out, n, sums, 1);
	return cudaGetLastError();
}

cudaError_t launch_max_u32(const uint32_t *in, size_t n, uint32_t *out, cudaStream_t s)
{
	cudaError_t e = cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
	if(e != cudaSuccess) return e;
	const unsigned nb = (unsigned) std::min<size_t>((n + 255) / 256 + 1, 4096);
	max_kernel<<<nb, 256, 0, s>>>(in, n, out);
	return cudaGetLastError();
}

cudaError_t launch_fan_count(const uint32_t *VT, const uint32_t *OT, const uint32_t *EVT, uint32_t nv,
                             uint32_t nhe, uint32_t *cnt, uint32_t *err, cudaStream_t s)
{
	if(!nv) return cudaSuccess;
	fan_count_kernel<<<(nv + 255) / 256, 256, 0, s>>>(VT, OT, EVT, nv, nhe, cnt, err);
	return cudaGetLastError();
}

// off[nv+1]: on entry the exclusive scan of the counts; on return bit 31 of
// off[v] carries the closed flag.  flags[nv] holds count | closed bit.
cudaError_t launch_fan_fill(const uint32_t *VT, const uint32_t *OT, const uint32_t *EVT, uint32_t nv,
                            const uint32_t *flags, uint32_t *off, uint32_t *fan, cudaStream_t s);

cudaError_t launch_fan_fill(const uint32_t *VT, const uint32_t *OT, const uint32_t *EVT, uint32_t nv,
                            const uint32_t *flags, uint32_t *off, uint32_t *fan, cudaStream_t s)
{
	if(!nv) return cudaSuccess;
	fan_fill_kernel<<<(nv + 255) / 256, 256, 0, s>>>(VT, OT, EVT, nv, flags, off, fan);
	return cudaGetLastError();
}

cudaError_t launch_fan8(const uint32_t *off, const uint32_t *fan, uint32_t nv, uint4 *rows, cudaStream_t s)
{
	if(!nv) return cudaSuccess;
	fan8_kernel<<<(nv + 255) / 256, 256, 0, s>>>(off, fan, nv, rows);
	return cudaGetLastError();
}

cudaError_t launch_mesh_stats(const uint32_t *VT, const uint32_t *OT, const float4 *pos, uint32_t nf, double *acc,
                              cudaStream_t s)
{
	if(!nf) return cudaSuccess;
	const unsigned nb = (unsigned) std::min<uint32_t>((nf + 255) / 256, 152 * 8);
	mesh_stats_kernel<<<nb, 256, 0, s>>>(VT, OT, pos, nf, acc);
	return cudaGetLastError();
}

cudaError_t launch_strip_flags(const uint32_t *in, uint32_t *out, uint32_t n, cudaStream_t s)
{
	if(!n) return cudaSuccess;
	strip_flag_kernel<<<(n + 255) / 256, 256, 0, s>>>(in, out, n);
	return cudaGetLastError();
}

cudaError_t launch_pos_convert(const double *xyz, uint32_t nv, float4 *pos, double *posd, cudaStream_t s)
{
	if(!nv) return cudaSuccess;
	pos_kernel<<<(nv + 255) / 256, 256, 0, s>>>(xyz, nv, pos, posd);
	return cudaGetLastError();
}

} // namespace gp
