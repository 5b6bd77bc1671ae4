// Toplesets (BFS rings) of many fields at once, on the GPU.
//
// Restates che::compute_toplesets (src/che.cpp:546-593) over the directed link
// relation che::link (src/che.cpp:102-112) so that ring indices, limits AND the
// order of `sorted` equal the reference's bit for bit.
//
// The reference appends a newly met vertex u the first time a ring-r vertex
// lists it, scanning ring r in `sorted` order and each link in link order.  So
// u's position in ring r+1 is fixed by the smallest key
// (position of the discovering vertex in `sorted`, slot in its link).
//
// One CTA owns one field at a time (fields are taken from a queue), so a level
// needs only CTA barriers:
//   discover: atomicMin(key[u], (pos << 20 | slot) + 1) for every link entry of
//             the frontier (no visited test, see discover());
//   emit:     frontier chunks in `sorted` order; each vertex counts the u
//             whose key it holds, a block scan (carried across chunks) gives
//             their positions, and the owners write them and set ring[u].
// The frontier's link rows stay in registers between the two passes and the
// frontier itself in shared memory, so a level costs two memory trips.
#include <mutex>

#include "gp_bfs.cuh"

namespace gp {

namespace {

#ifndef GP_BT
#define GP_BT 1024
#endif
constexpr int BT = GP_BT;  // threads of a BFS CTA

// Frontier vertices whose link rows a thread keeps in registers between the
// two passes of a level, and the shared-memory copy of the frontier.
#ifndef GP_KB
#define GP_KB 1
#endif
constexpr uint32_t KB = GP_KB;
constexpr uint32_t SF = BT * KB;

__global__ void __launch_bounds__(BT, 1) bfs_kernel(FieldDev *fields, FieldState *state, uint32_t n_fields,
                                                 uint32_t *queue, const uint32_t *order)
{
	__shared__ uint32_t s_f;
	__shared__ uint32_t sf[2][SF];  // frontier copies: current and next level
	for(;;)
	{
		if(threadIdx.x == 0) s_f = atomicAdd(queue, 1u);
		__syncthreads();
		const uint32_t ticket = s_f;
		__syncthreads();
		if(ticket >= n_fields) return;
		const uint32_t f = order ? order[ticket] : ticket;
		const FieldDev &F = fields[f];
		if(!state[f].bfs_live || F.stream) continue;  // no sources, a source out of range, or streamed

		uint32_t level = 0, s = 0, e = F.ns;  // frontier = ring 0 = [0, ns)
		uint32_t cur = 0;
		bool in_smem = false;                 // ring 0 is read from `sorted`
		for(;;)
		{
			// pass 1: rows of the frontier (first KB chunks kept in registers), discover
			uint4 ra[KB], rb[KB];
			uint32_t vv[KB], cm[KB];
#pragma unroll
			for(uint32_t c = 0; c < KB; c++)
			{
				const uint32_t p = s + c * BT + threadIdx.x;
				if(p < e)
				{
					vv[c] = in_smem ? sf[cur][p - s] : ldcg(F.sorted + p);
					ra[c] = __ldg(F.m.fan8 + 2 * (size_t) vv[c]);
					rb[c] = __ldg(F.m.fan8 + 2 * (size_t) vv[c] + 1);
					cm[c] = discover_local(F, p, vv[c], ra[c], rb[c]);
				}
			}
			for(uint32_t p = s + SF + threadIdx.x; p < e; p += BT)
			{
				const uint32_t v = ldcg(F.sorted + p);
				discover_local(F, p, v, __ldg(F.m.fan8 + 2 * (size_t) v), __ldg(F.m.fan8 + 2 * (size_t) v + 1));
			}
			__syncthreads();
			// pass 2: count, scan in frontier order (carried across chunks), emit
			uint32_t carry = 0;
			for(uint32_t base = s, c = 0; base < e; base += BT, c++)
			{
				const uint32_t p = base + threadIdx.x;
				uint32_t v = 0, cnt = 0, mask = 0, cand = 0xFFu;
				uint4 a = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY), b = a;
				if(p < e)
				{
					if(c < KB)
					{
						// registers of pass 1 (the loops unroll, so c is a constant per copy)
#pragma unroll
						for(uint32_t k = 0; k < KB; k++)
							if(k == c)
							{
								v = vv[k];
								a = ra[k];
								b = rb[k];
								cand = cm[k];
							}
					}
					else
					{
						v = ldcg(F.sorted + p);
						a = __ldg(F.m.fan8 + 2 * (size_t) v);
						b = __ldg(F.m.fan8 + 2 * (size_t) v + 1);
					}
					mask = owned(F, p, v, a, b, cnt, cand);
				}
				uint32_t tot;
				const uint32_t ex = block_exclusive_scan<BT>(cnt, &tot);
				if(cnt)
				{
					uint32_t o = carry + ex;
					if(b.w == FAN8_OVERFLOW)
					{
						const uint32_t o0 = __ldg(F.m.fan_off + v) & FAN_MASK, o1 = __ldg(F.m.fan_off + v + 1) & FAN_MASK;
						for(uint32_t q = o0; q < o1; q++)
						{
							const uint32_t u = __ldg(F.m.fan + q);
							if(ldcg(F.key + u) == (((unsigned long long) p << 20) | (q - o0)) + 1)
							{
								F.sorted[e + o] = u;
								F.ring[u] = level + 1;
								if(F.inv) F.inv[u] = e + o + 1;
								if(o < SF) sf[cur ^ 1][o] = u;
								o++;
							}
						}
					}
					else
#pragma unroll
						for(uint32_t q = 0; q < 8; q++)
							if(mask & (1u << q))
							{
								const uint32_t u = slot_of(a, b, q);
								F.sorted[e + o] = u;
								F.ring[u] = level + 1;
								if(F.inv) F.inv[u] = e + o + 1;
								if(o < SF) sf[cur ^ 1][o] = u;
								o++;
							}
				}
				carry += tot;
			}
			__syncthreads();
			if(!carry) break;
			if(threadIdx.x == 0) F.limits[level + 2] = e + carry;
			in_smem = carry <= SF;
			cur ^= 1;
			s = e;
			e += carry;
			level++;
		}
		if(threadIdx.x == 0)
		{
			state[f].n_limits = level + 2;
			state[f].bfs_live = 0;
		}
		__syncthreads();
	}
}

// ---------------------------------------------------------------------------
// Wide fields: every CTA of one cooperative launch works on each level of one
// field (fields taken one after another).  For a field on a large mesh with
// many sources (farthest-point sampling: hundreds of sources on millions of
// vertices) a level holds tens of thousands of vertices, more than one CTA
// can turn over quickly.  A level costs two grid barriers:
//   [barrier] count: the frontier is cut into one contiguous chunk per CTA;
//             each CTA counts the vertices its chunk owns (key match);
//   [barrier] emit:  each CTA adds up the counts of the CTAs before it, writes
//             its owned vertices in frontier order, and at once discovers
//             their neighbours for the next level (it knows their positions).
// Discovering level L+2 while other CTAs still emit level L+1 is safe: those
// keys carry positions past every level-L+1 key, so they never lower a key a
// level-L+1 owner compares against, and only reach vertices not yet met.
// ---------------------------------------------------------------------------
constexpr int BG = 1024;  // threads of a wide-BFS CTA

// Counting barrier over the whole launch (bar[0] arrivals, bar[1] abort,
// bar[2] error bits); gives up after SPIN_LIMIT polls.
__device__ __forceinline__ bool bfs_grid_barrier(uint32_t *bar, uint32_t target)
{
	__shared__ uint32_t s_ok;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		s_ok = 1;
		asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
		uint32_t spins = 0;
		while(ld_acquire(bar) < target)
		{
			if(++spins > SPIN_LIMIT || ld_relaxed(bar + 1))
			{
				atomicOr(bar + 2, DEV_ERR_TIMEOUT);
				atomicExch(bar + 1, 1u);
				s_ok = 0;
				break;
			}
		}
	}
	__syncthreads();
	return s_ok != 0;
}

__device__ __forceinline__ void load_row(const FieldDev &F, uint32_t v, uint4 &a, uint4 &b)
{
	a = __ldg(F.m.fan8 + 2 * (size_t) v);
	b = __ldg(F.m.fan8 + 2 * (size_t) v + 1);
}

// Emit the vertices owned by frontier position p (key match) at sorted[o...]
// in link order, set their ring, and discover their neighbours.
__device__ __forceinline__ void emit_owned(const FieldDev &F, uint32_t p, uint32_t v, const uint4 &a, const uint4 &b,
                                           uint32_t mask, uint32_t o, uint32_t level)
{
	auto put = [&](uint32_t u) {
		F.sorted[o] = u;
		F.ring[u] = level + 1;
		if(F.inv) F.inv[u] = o + 1;
		uint4 ua, ub;
		load_row(F, u, ua, ub);
		discover(F, o, u, ua, ub);
		o++;
	};
	if(b.w == FAN8_OVERFLOW)
	{
		const uint32_t o0 = __ldg(F.m.fan_off + v) & FAN_MASK, o1 = __ldg(F.m.fan_off + v + 1) & FAN_MASK;
		for(uint32_t q = o0; q < o1; q++)
		{
			const uint32_t u = __ldg(F.m.fan + q);
			if(ldcg(F.key + u) == (((unsigned long long) p << 20) | (q - o0)) + 1) put(u);
		}
		return;
	}
#pragma unroll
	for(uint32_t q = 0; q < 8; q++)
		if(mask & (1u << q)) put(slot_of(a, b, q));
}

__global__ void __launch_bounds__(BG, 1) bfs_grid_kernel(FieldDev *fields, FieldState *state, const uint32_t *wide,
                                                      uint32_t n_wide, uint32_t *bar, uint32_t *cta_tot)
{
	__shared__ uint32_t s_pre, s_tot;
	const uint32_t G = gridDim.x, b = blockIdx.x;
	const uint32_t gt = b * BG + threadIdx.x, gn = G * BG;
	uint32_t nbar = 0;
	for(uint32_t w = 0; w < n_wide; w++)
	{
		const uint32_t f = wide[w];
		const FieldDev &F = fields[f];
		if(!state[f].bfs_live) continue;  // no sources, or a source out of range (uniform)
		// level 0: the sources (ring 0) discover their neighbours
		for(uint32_t p = gt; p < F.ns; p += gn)
		{
			const uint32_t v = ldcg(F.sorted + p);
			uint4 ra, rb;
			load_row(F, v, ra, rb);
			discover(F, p, v, ra, rb);
		}
		uint32_t level = 0, s = 0, e = F.ns;
		for(;;)
		{
			if(!bfs_grid_barrier(bar, G * ++nbar)) return;
			const uint32_t n = e - s, chunk = (n + G - 1) / G;
			const uint32_t c0 = s + min(n, b * chunk), c1 = s + min(n, (b + 1) * chunk);
			// count this CTA's owned vertices; the first round's rows and masks stay in registers
			uint32_t v0 = 0, m0 = 0, n0 = 0, tot = 0;
			uint4 a0 = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY), b0 = a0;
			for(uint32_t base = c0; base < c1; base += BG)
			{
				const uint32_t p = base + threadIdx.x;
				uint32_t cnt = 0;
				if(p < c1)
				{
					uint32_t v = ldcg(F.sorted + p), mask;
					uint4 ra, rb;
					load_row(F, v, ra, rb);
					mask = owned(F, p, v, ra, rb, cnt);
					if(base == c0)
					{
						v0 = v;
						a0 = ra;
						b0 = rb;
						m0 = mask;
						n0 = cnt;
					}
				}
				uint32_t t;
				block_exclusive_scan<BG>(cnt, &t);
				tot += t;
			}
			if(threadIdx.x == 0) cta_tot[b] = tot;
			if(!bfs_grid_barrier(bar, G * ++nbar)) return;
			// offset of this CTA's chunk and the level's total
			if(threadIdx.x == 0)
			{
				s_pre = 0;
				s_tot = 0;
			}
			__syncthreads();
			{
				uint32_t pre = 0, all = 0;
				for(uint32_t k = threadIdx.x; k < G; k += BG)
				{
					const uint32_t x = ldcg(cta_tot + k);
					all += x;
					if(k < b) pre += x;
				}
				if(pre) atomicAdd(&s_pre, pre);
				if(all) atomicAdd(&s_tot, all);
			}
			__syncthreads();
			const uint32_t grand = s_tot;
			if(!grand) break;
			uint32_t carry = e + s_pre;
			for(uint32_t base = c0; base < c1; base += BG)
			{
				const uint32_t p = base + threadIdx.x;
				uint32_t v = 0, mask = 0, cnt = 0;
				uint4 ra = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY), rb = ra;
				if(p < c1)
				{
					if(base == c0)
					{
						v = v0;
						ra = a0;
						rb = b0;
						mask = m0;
						cnt = n0;
					}
					else
					{
						v = ldcg(F.sorted + p);
						load_row(F, v, ra, rb);
						mask = owned(F, p, v, ra, rb, cnt);
					}
				}
				uint32_t t;
				const uint32_t ex = block_exclusive_scan<BG>(cnt, &t);
				if(cnt) emit_owned(F, p, v, ra, rb, mask, carry + ex, level);
				carry += t;
			}
			if(b == 0 && threadIdx.x == 0) F.limits[level + 2] = e + grand;
			s = e;
			e += grand;
			level++;
		}
		if(b == 0 && threadIdx.x == 0)
		{
			state[f].n_limits = level + 2;
			state[f].bfs_live = 0;
		}
	}
}

// Per-field setup: ring = NIL, key = max over the field's vertices.
__global__ void bfs_clear_kernel(FieldDev *fields, const uint32_t *vbase, uint32_t n_fields, uint32_t total)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(vbase, n_fields, g);
		const uint32_t v = g - vbase[f];
		fields[f].ring[v] = NIL;
		fields[f].key[v] = ~0ull;
		if(fields[f].inv) fields[f].inv[v] = 0;  // position + 1 of v, 0: unreached
	}
}

// Sources -> ring 0, in the order given (duplicates kept, src/che.cpp:555-561).
__global__ void bfs_seed_kernel(FieldDev *fields, FieldState *state, uint32_t n_fields)
{
	const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
	if(f >= n_fields) return;
	FieldDev &F = fields[f];
	FieldState &st = state[f];
	st.status = 0;
	for(uint32_t s = 0; s < F.ns; s++)
		if(F.src[s] >= F.m.nv)
		{
			// a source outside the mesh: report it and leave the field empty
			st.status = DEV_ERR_BOUNDS;
			st.bfs_live = 0;
			st.n_limits = 0;
			return;
		}
	for(uint32_t s = 0; s < F.ns; s++)
	{
		const uint32_t v = F.src[s];
		F.sorted[s] = v;
		F.ring[v] = 0;
		F.key[v] = 0;  // below every discovery key: a source is never re-discovered
		if(F.inv) F.inv[v] = s + 1;  // repeated sources: the last occurrence
	}
	F.limits[0] = 0;
	F.limits[1] = F.ns;
	st.bfs_live = F.ns > 0;
	st.n_limits = F.ns > 0 ? 2 : 0;
}

} // namespace

cudaError_t launch_bfs_setup(FieldDev *fields, FieldState *state, const uint32_t *vbase, uint32_t n_fields,
                             uint32_t total_vertices, cudaStream_t s)
{
	if(total_vertices)
	{
		const unsigned nb = (unsigned) std::min<uint32_t>((total_vertices + 255) / 256, 152 * 16);
		bfs_clear_kernel<<<nb, 256, 0, s>>>(fields, vbase, n_fields, total_vertices);
	}
	bfs_seed_kernel<<<(n_fields + 127) / 128, 128, 0, s>>>(fields, state, n_fields);
	return cudaGetLastError();
}

int toplesets_max_ctas(int device)
{
	int nsm = 0, per = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, bfs_kernel, BT, 0);
	return nsm * per;
}

int toplesets_wide_ctas(int device)
{
	int nsm = 0, per = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, bfs_grid_kernel, BG, 0);
	return nsm * std::max(per, 0);
}

// wide: the fields (ids) run by the cooperative launch, n_wide of them;
// bar: 4 words, zeroed here; cta_tot: ctas words.
cudaError_t launch_toplesets_wide(FieldDev *fields, FieldState *state, const uint32_t *wide, uint32_t n_wide,
                                  uint32_t *bar, uint32_t *cta_tot, uint32_t ctas, cudaStream_t s)
{
	if(!n_wide || !ctas) return cudaSuccess;
	cudaError_t e = cudaMemsetAsync(bar, 0, 4 * sizeof(uint32_t), s);
	if(e != cudaSuccess) return e;
	void *args[] = {&fields, &state, &wide, &n_wide, &bar, &cta_tot};
	return cudaLaunchCooperativeKernel((const void *) bfs_grid_kernel, dim3(ctas), dim3(BG), args, 0, s);
}

// queue: one word, zeroed here (the field ticket); order: the fields in the
// order the CTAs take them (null: by index)
cudaError_t launch_toplesets(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *queue,
                             uint32_t ctas, const uint32_t *order, cudaStream_t s)
{
	cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
	if(e != cudaSuccess) return e;
	ctas = std::max<uint32_t>(1, std::min<uint32_t>(ctas, n_fields));
	bfs_kernel<<<ctas, BT, 0, s>>>(fields, state, n_fields, queue, order);
	return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Toplesets without any device allocation (gp_toplesets_noalloc).
//
// Some callers may not allocate device memory while they compute: an
// application that has handed all device memory to its own pool up front, or
// a latency-critical loop in which cudaMalloc/cudaFree (which can stall the
// whole device) are not allowed.  For them the BFS scratch -- the per-vertex
// discovery keys and the small field descriptor -- lives in one fixed
// file-scope device array instead of the context workspace.  Every GPU that
// loads this library reserves that array until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t NOALLOC_MAX_VERTICES = 1u << 20;  // largest mesh the array serves
constexpr size_t NOALLOC_HEADER = 4096;               // field descriptor, state, queue

struct NoallocHeader {
	FieldDev f;
	FieldState st;
	uint32_t vbase[2];
	uint32_t queue;
};
static_assert(sizeof(NoallocHeader) <= NOALLOC_HEADER, "header size");

// header, then 8-byte keys for up to NOALLOC_MAX_VERTICES vertices (about 8 MiB)
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_HEADER + 8ull * NOALLOC_MAX_VERTICES];

// Writes this call's descriptor into the array and clears what must start at
// zero (the queue ticket and the field state); the keys are reset by
// bfs_clear_kernel.  Earlier calls' contents are otherwise left in place.
__global__ void noalloc_setup_kernel(MeshDev m, const uint32_t *src, uint32_t ns, uint32_t *rings, uint32_t *sorted,
                                     uint32_t cap_sorted, uint32_t *limits)
{
	if(threadIdx.x != 0) return;
	NoallocHeader *h = reinterpret_cast<NoallocHeader *>(g_noalloc_scratch);
	FieldDev f;
	memset(&f, 0, sizeof(f));
	f.m = m;
	f.src = src;
	f.ns = ns;
	f.cap_sorted = cap_sorted;
	f.ring = rings;
	f.key = reinterpret_cast<unsigned long long *>(g_noalloc_scratch + NOALLOC_HEADER);
	f.sorted = sorted;
	f.limits = limits;
	h->f = f;
	memset(&h->st, 0, sizeof(h->st));
	h->vbase[0] = 0;
	h->vbase[1] = m.nv;
	h->queue = 0;
}

__global__ void noalloc_finish_kernel(uint32_t *n_limits)
{
	if(threadIdx.x != 0) return;
	const NoallocHeader *h = reinterpret_cast<const NoallocHeader *>(g_noalloc_scratch);
	*n_limits = h->st.status ? 0u : h->st.n_limits;
}

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};

// Device address of the array on the current device (the symbol's host-side
// name is not a device address).  Looked up again on every call made outside
// stream capture, so that a device reset between calls (which unloads and
// reloads this module) never leaves a stale address; a call made while `s` is
// being captured reuses the address of the last uncaptured call on the device.
gp_status noalloc_scratch(cudaStream_t s, void **out)
{
	int dev = -1;
	if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
	{
		cudaGetLastError();
		return GP_ERR_NO_DEVICE;
	}
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	if(cudaStreamIsCapturing(s, &cs) != cudaSuccess)
	{
		cudaGetLastError();
		cs = cudaStreamCaptureStatusActive;  // cannot tell: treat as capturing
	}
	std::lock_guard<std::mutex> lock(g_noalloc_mu);
	if(cs == cudaStreamCaptureStatusNone)
	{
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if(e != cudaSuccess || !p)
		{
			cudaGetLastError();
			return GP_ERR_CUDA;
		}
		g_noalloc_ptr[dev] = p;
	}
	else if(!g_noalloc_ptr[dev])
		return GP_ERR_INVALID_ARG;  // the first call on a device must come before any capture
	*out = g_noalloc_ptr[dev];
	return GP_OK;
}

} // namespace

} // namespace gp

extern "C" gp_status gp_toplesets_noalloc(const gp_mesh *mesh, const uint32_t *sources, uint32_t n_sources,
                                          uint32_t *rings, uint32_t *sorted, uint32_t cap_sorted, uint32_t *limits,
                                          uint32_t cap_limits, uint32_t *n_limits, void *stream)
{
	using namespace gp;
	if(!mesh || !sources || !n_sources || !rings || !sorted || !limits || !n_limits) return GP_ERR_INVALID_ARG;
	const MeshDev *m = mesh_dev(mesh);
	if(m->nv > NOALLOC_MAX_VERTICES) return GP_ERR_CAPACITY;  // the fixed array holds 2^20 vertices
	if((uint64_t) cap_sorted < (uint64_t) m->nv + n_sources || (uint64_t) cap_limits < (uint64_t) m->nv + 2)
		return GP_ERR_CAPACITY;
	int dev = -1;
	if(cudaGetDevice(&dev) != cudaSuccess || dev != mesh_device(mesh))
	{
		cudaGetLastError();
		return GP_ERR_INVALID_ARG;  // the mesh's device must be current
	}
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	void *base = nullptr;
	const gp_status st = noalloc_scratch(s, &base);
	if(st != GP_OK) return st;
	NoallocHeader *h = static_cast<NoallocHeader *>(base);
	noalloc_setup_kernel<<<1, 32, 0, s>>>(*m, sources, n_sources, rings, sorted, cap_sorted, limits);
	bfs_clear_kernel<<<(unsigned) std::min<uint32_t>((m->nv + 255) / 256, 152 * 16), 256, 0, s>>>(&h->f, h->vbase, 1,
	                                                                                              m->nv);
	bfs_seed_kernel<<<1, 32, 0, s>>>(&h->f, &h->st, 1);
	bfs_kernel<<<1, BT, 0, s>>>(&h->f, &h->st, 1, &h->queue, nullptr);
	noalloc_finish_kernel<<<1, 32, 0, s>>>(n_limits);
	return cudaGetLastError() == cudaSuccess ? GP_OK : GP_ERR_CUDA;
}

