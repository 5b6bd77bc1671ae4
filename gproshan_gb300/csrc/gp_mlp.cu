// Learned sweep-cost model: a 3-layer MLP (N_IN -> 64 -> 64 -> 2, ReLU) with
// hand-written FP32 training kernels (forward, backward, Adam) and BF16
// tensor-core inference (mma.sync m16n8k16, FP32 accumulation).
//
// It predicts, per field, log(sweeps / rings) and log(relaxations / vertices)
// from features of the field's toplesets and mesh.  The batch scheduler uses
// the prediction only to decide where a field starts and in which order fields
// are taken; it never changes which sweeps run, so results are identical with
// or without it (the reference's schedule is reproduced exactly either way).
//
// Parameter layout (floats): W1[N_IN][H] b1[H] W2[H][H] b2[H] W3[H][N_OUT] b3[N_OUT].
#include <cuda_bf16.h>

#include "gp_common.cuh"
#include "gp_mlp.h"

namespace gp {

namespace {

constexpr int NI = MLP_IN, NH = MLP_H, NO = MLP_OUT;
constexpr int OW1 = 0, OB1 = OW1 + NI * NH, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NH * NO, NPARAM = OB3 + NO;
static_assert(NPARAM == MLP_NPARAM, "layout");

// ---- FP32 forward: one thread per (sample, unit) --------------------------
__global__ void dense_relu(const float *__restrict__ X, int n, int k, const float *__restrict__ W,
                           const float *__restrict__ b, int m, float *__restrict__ Y, int relu)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n * m) return;
	const int r = i / m, c = i % m;
	float s = b[c];
	for(int q = 0; q < k; q++) s = fmaf(X[r * k + q], W[q * m + c], s);
	Y[i] = relu ? fmaxf(s, 0.f) : s;
}

// dY = 2 (Y - T) / (n * NO) (mean squared error over all outputs), loss partial sums
__global__ void mse_grad(const float *__restrict__ Y, const float *__restrict__ T, int n, float *__restrict__ dY,
                         float *__restrict__ loss)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	float l = 0.f;
	if(i < n * NO)
	{
		const float e = Y[i] - T[i];
		dY[i] = 2.f * e / (float) (n * NO);
		l = e * e / (float) (n * NO);
	}
	for(int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
	if((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// dX[r][q] = sum_c dY[r][c] W[q][c], masked by ReLU of the layer that made X
__global__ void back_input(const float *__restrict__ dY, int n, int m, const float *__restrict__ W, int k,
                           const float *__restrict__ Xact, float *__restrict__ dX)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n * k) return;
	const int r = i / k, q = i % k;
	float s = 0.f;
	for(int c = 0; c < m; c++) s = fmaf(dY[r * m + c], W[q * m + c], s);
	dX[i] = Xact[i] > 0.f ? s : 0.f;
}

// dW[q][c] = sum_r X[r][q] dY[r][c]; db[c] = sum_r dY[r][c]  (one thread per weight)
__global__ void back_weights(const float *__restrict__ X, const float *__restrict__ dY, int n, int k, int m,
                             float *__restrict__ dW, float *__restrict__ db)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < k * m)
	{
		const int q = i / m, c = i % m;
		float s = 0.f;
		for(int r = 0; r < n; r++) s = fmaf(X[r * k + q], dY[r * m + c], s);
		dW[i] = s;
	}
	else if(i < k * m + m)
	{
		const int c = i - k * m;
		float s = 0.f;
		for(int r = 0; r < n; r++) s += dY[r * m + c];
		db[c] = s;
	}
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                            float *__restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const float gi = g[i];
	const float a = b1 * m1[i] + (1.f - b1) * gi;
	const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
	m1[i] = a;
	m2[i] = b;
	p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// ---- BF16 tensor-core inference ---------------------------------------------
// One warp evaluates 16 samples.  m16n8k16 fragments (PTX ISA, mma.m16n8k16
// .bf16): with g = lane/4, t = lane%4, A (16x16, row-major) holds
// {A[g][2t..2t+1], A[g+8][2t..], A[g][2t+8..], A[g+8][2t+8..]}, B (16x8,
// column) holds {B[2t..2t+1][g], B[2t+8..][g]}, and C (16x8, f32) holds
// {C[g][2t], C[g][2t+1], C[g+8][2t], C[g+8][2t+1]}.  The C fragments of
// n-tiles 2q and 2q+1 are exactly the A fragment of k-step q of the next
// layer, so activations never leave registers.
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
	const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1)
{
	asm volatile(
	    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	    "{%0,%1,%2,%3};"
	    : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
	    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// B fragment of weights W[k][n] (row-major K x N) for k-step ks, n-tile nt
__device__ __forceinline__ void load_b(const __nv_bfloat16 *W, int N, int ks, int nt, int g, int t, uint32_t &b0,
                                       uint32_t &b1)
{
	const int k0 = ks * 16 + 2 * t, n = nt * 8 + g;
	__nv_bfloat162 x, y;
	x.x = W[(k0) * N + n];
	x.y = W[(k0 + 1) * N + n];
	y.x = W[(k0 + 8) * N + n];
	y.y = W[(k0 + 9) * N + n];
	b0 = *reinterpret_cast<uint32_t *>(&x);
	b1 = *reinterpret_cast<uint32_t *>(&y);
}

// Weights converted to BF16 once per launch into shared memory (W3 padded to 8 columns).
__global__ void __launch_bounds__(128) mlp_infer_bf16(const float *__restrict__ P, const float *__restrict__ X, int n,
                                                      float *__restrict__ Y)
{
	__shared__ __nv_bfloat16 w1[NI * NH], w2[NH * NH], w3[NH * 8];
	__shared__ float bb1[NH], bb2[NH], bb3[8];
	for(int i = threadIdx.x; i < NI * NH; i += blockDim.x) w1[i] = __float2bfloat16_rn(P[OW1 + i]);
	for(int i = threadIdx.x; i < NH * NH; i += blockDim.x) w2[i] = __float2bfloat16_rn(P[OW2 + i]);
	for(int i = threadIdx.x; i < NH * 8; i += blockDim.x)
	{
		const int r = i / 8, c = i % 8;
		w3[i] = __float2bfloat16_rn(c < NO ? P[OW3 + r * NO + c] : 0.f);
	}
	for(int i = threadIdx.x; i < NH; i += blockDim.x)
	{
		bb1[i] = P[OB1 + i];
		bb2[i] = P[OB2 + i];
	}
	if(threadIdx.x < 8) bb3[threadIdx.x] = threadIdx.x < NO ? P[OB3 + threadIdx.x] : 0.f;
	__syncthreads();

	const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	const int row0 = (blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)) * 16;
	if(row0 >= n) return;  // whole warp leaves together
	auto xin = [&](int r, int c) { return r < n ? X[r * NI + c] : 0.f; };
	// layer 1: A = X (16 x NI, one k-step), 8 n-tiles
	uint32_t a[4] = {pack_bf16(xin(row0 + g, 2 * t), xin(row0 + g, 2 * t + 1)),
	                 pack_bf16(xin(row0 + g + 8, 2 * t), xin(row0 + g + 8, 2 * t + 1)),
	                 pack_bf16(xin(row0 + g, 2 * t + 8), xin(row0 + g, 2 * t + 9)),
	                 pack_bf16(xin(row0 + g + 8, 2 * t + 8), xin(row0 + g + 8, 2 * t + 9))};
	float h[8][4];
#pragma unroll
	for(int nt = 0; nt < 8; nt++)
	{
		const float c0 = bb1[nt * 8 + 2 * t], c1 = bb1[nt * 8 + 2 * t + 1];
		h[nt][0] = c0;
		h[nt][1] = c1;
		h[nt][2] = c0;
		h[nt][3] = c1;
		uint32_t b0, b1;
		load_b(w1, NH, 0, nt, g, t, b0, b1);
		mma_bf16(h[nt], a, b0, b1);
	}
	// layer 2: A fragments from the ReLU'd accumulators, 4 k-steps x 8 n-tiles
	uint32_t a2[4][4];
#pragma unroll
	for(int q = 0; q < 4; q++)
	{
		a2[q][0] = pack_bf16(fmaxf(h[2 * q][0], 0.f), fmaxf(h[2 * q][1], 0.f));
		a2[q][1] = pack_bf16(fmaxf(h[2 * q][2], 0.f), fmaxf(h[2 * q][3], 0.f));
		a2[q][2] = pack_bf16(fmaxf(h[2 * q + 1][0], 0.f), fmaxf(h[2 * q + 1][1], 0.f));
		a2[q][3] = pack_bf16(fmaxf(h[2 * q + 1][2], 0.f), fmaxf(h[2 * q + 1][3], 0.f));
	}
#pragma unroll
	for(int nt = 0; nt < 8; nt++)
	{
		const float c0 = bb2[nt * 8 + 2 * t], c1 = bb2[nt * 8 + 2 * t + 1];
		h[nt][0] = c0;
		h[nt][1] = c1;
		h[nt][2] = c0;
		h[nt][3] = c1;
#pragma unroll
		for(int q = 0; q < 4; q++)
		{
			uint32_t b0, b1;
			load_b(w2, NH, q, nt, g, t, b0, b1);
			mma_bf16(h[nt], a2[q], b0, b1);
		}
	}
	// layer 3: one n-tile of 8 (NO used)
#pragma unroll
	for(int q = 0; q < 4; q++)
	{
		a2[q][0] = pack_bf16(fmaxf(h[2 * q][0], 0.f), fmaxf(h[2 * q][1], 0.f));
		a2[q][1] = pack_bf16(fmaxf(h[2 * q][2], 0.f), fmaxf(h[2 * q][3], 0.f));
		a2[q][2] = pack_bf16(fmaxf(h[2 * q + 1][0], 0.f), fmaxf(h[2 * q + 1][1], 0.f));
		a2[q][3] = pack_bf16(fmaxf(h[2 * q + 1][2], 0.f), fmaxf(h[2 * q + 1][3], 0.f));
	}
	float o[4] = {bb3[2 * t], bb3[2 * t + 1], bb3[2 * t], bb3[2 * t + 1]};
#pragma unroll
	for(int q = 0; q < 4; q++)
	{
		uint32_t b0, b1;
		load_b(w3, 8, q, 0, g, t, b0, b1);
		mma_bf16(o, a2[q], b0, b1);
	}
	// columns 2t, 2t+1 of rows g, g+8: only t == 0 holds the NO = 2 outputs
	if(t == 0)
	{
		if(row0 + g < n)
		{
			Y[(row0 + g) * NO] = o[0];
			Y[(row0 + g) * NO + 1] = o[1];
		}
		if(row0 + g + 8 < n)
		{
			Y[(row0 + g + 8) * NO] = o[2];
			Y[(row0 + g + 8) * NO + 1] = o[3];
		}
	}
}

unsigned nb(long n, int t = 256) { return (unsigned) ((n + t - 1) / t); }

} // namespace

size_t mlp_workspace_floats(int n)
{
	// activations H1, H2, output Y, dY, dH2, dH1, gradients, Adam moments, loss
	return (size_t) n * (NH + NH + NO + NO + NH + NH) + 3 * (size_t) NPARAM + 64;
}

// One forward + backward pass: grads (NPARAM) and *loss (device) from params.
cudaError_t mlp_grad_device(const float *P, const float *X, const float *T, int n, float *work, float *grads,
                            float *loss, cudaStream_t s)
{
	float *H1 = work, *H2 = H1 + (size_t) n * NH, *Yo = H2 + (size_t) n * NH, *dY = Yo + (size_t) n * NO;
	float *dH2 = dY + (size_t) n * NO, *dH1 = dH2 + (size_t) n * NH;
	cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(float), s);
	if(e != cudaSuccess) return e;
	dense_relu<<<nb((long) n * NH), 256, 0, s>>>(X, n, NI, P + OW1, P + OB1, NH, H1, 1);
	dense_relu<<<nb((long) n * NH), 256, 0, s>>>(H1, n, NH, P + OW2, P + OB2, NH, H2, 1);
	dense_relu<<<nb((long) n * NO), 256, 0, s>>>(H2, n, NH, P + OW3, P + OB3, NO, Yo, 0);
	mse_grad<<<nb((long) n * NO), 256, 0, s>>>(Yo, T, n, dY, loss);
	back_weights<<<nb(NH * NO + NO), 256, 0, s>>>(H2, dY, n, NH, NO, grads + OW3, grads + OB3);
	back_input<<<nb((long) n * NH), 256, 0, s>>>(dY, n, NO, P + OW3, NH, H2, dH2);
	back_weights<<<nb(NH * NH + NH), 256, 0, s>>>(H1, dH2, n, NH, NH, grads + OW2, grads + OB2);
	back_input<<<nb((long) n * NH), 256, 0, s>>>(dH2, n, NH, P + OW2, NH, H1, dH1);
	back_weights<<<nb(NI * NH + NH), 256, 0, s>>>(X, dH1, n, NI, NH, grads + OW1, grads + OB1);
	return cudaGetLastError();
}

cudaError_t mlp_forward_f32_device(const float *P, const float *X, int n, float *work, float *Y, cudaStream_t s)
{
	float *H1 = work, *H2 = H1 + (size_t) n * NH;
	dense_relu<<<nb((long) n * NH), 256, 0, s>>>(X, n, NI, P + OW1, P + OB1, NH, H1, 1);
	dense_relu<<<nb((long) n * NH), 256, 0, s>>>(H1, n, NH, P + OW2, P + OB2, NH, H2, 1);
	dense_relu<<<nb((long) n * NO), 256, 0, s>>>(H2, n, NH, P + OW3, P + OB3, NO, Y, 0);
	return cudaGetLastError();
}

cudaError_t mlp_infer_bf16_device(const float *P, const float *X, int n, float *Y, cudaStream_t s)
{
	if(n <= 0) return cudaSuccess;
	const int warps = (n + 15) / 16;
	mlp_infer_bf16<<<(warps + 3) / 4, 128, 0, s>>>(P, X, n, Y);
	return cudaGetLastError();
}

cudaError_t mlp_adam_device(float *P, const float *grads, float *m1, float *m2, float lr, int step, cudaStream_t s)
{
	const float b1 = 0.9f, b2 = 0.999f;
	const float c1 = 1.f - powf(b1, (float) step), c2 = 1.f - powf(b2, (float) step);
	adam_kernel<<<nb(NPARAM), 256, 0, s>>>(P, grads, m1, m2, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
	return cudaGetLastError();
}

} // namespace gp
