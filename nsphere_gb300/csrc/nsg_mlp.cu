// nsg_mlp.cu -- the learned level scheduler: a 4 -> 64 -> 64 -> 8 MLP that predicts
// the adaptive-leapfrog level a particle will accept, with BF16 weights, FP32
// accumulation, hand-written inference and training kernels on the tensor cores:
// inference (the part that runs every learned step) on the fifth-generation tensor
// cores (tcgen05.mma with the accumulators in tensor memory, nsg_tc.cuh), 128
// particles per MMA; training (a few small launches per epoch) with mma.sync
// m16n8k16 warp tiles.
//
// Inputs per particle (FP32, computed from the state as the step starts, in its array
// order -- the previous sort's -- whose position stands for the rank):
//   x0 = log2(r) / 8
//   x1 = clamp(v_r / v_c, -8, 8) / 4          v_c = sqrt(-gnum / r) = sqrt(G M_i / r)
//   x2 = log2(|ell| / (r v_c) + 1e-6) / 8     circularity
//   x3 = log2(dt / t_dyn) / 8                 local dynamical time t_dyn = r / v_c
// Output: softmax over 8 classes, class k = accepted level k (7 also = never).
//
// Prediction never changes a result: in learned mode a particle predicted to need
// level >= 1 skips the level-0 pass (k_fused_level0, or k_gather_level0 on the
// two-kernel path) and goes straight to the level-parallel kernel, which still tests
// every level from 0 upward in the reference's order (the plain error test judges
// every particle).
//
// Weight layout (float master copy and bf16 copy, row-major [out][in]):
//   W1 [64][16] (inputs 4..15 zero), b1[64], W2 [64][64], b2[64], W3 [8][64], b3[8].
#include <cuda_bf16.h>

#include "nsg_internal.cuh"
#include "nsg_tc.cuh"

namespace nsg {

constexpr int kH = 64, kIn = 16, kOut = 8;
constexpr int kW1 = kH * kIn, kW2 = kH * kH, kW3 = kOut * kH;
constexpr int kOffW1 = 0, kOffB1 = kW1, kOffW2 = kOffB1 + kH, kOffB2 = kOffW2 + kW2,
              kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kW3, kParams = kOffB3 + kOut;
// biases staged compactly in shared memory: b1 [0, 64), b2 [64, 128), b3 [128, 136)
constexpr int kBB1 = 0, kBB2 = kH, kBB3 = 2 * kH, kBias = 2 * kH + kOut;

struct MlpDev {
    float *w = nullptr;        // [kParams] master weights
    float *g = nullptr;        // [kParams] gradient accumulator
    float *m = nullptr, *v = nullptr;  // Adam moments
    __nv_bfloat16 *wb = nullptr;       // bf16 copies of W1, W2, W3 (same offsets, biases unused)
    float *feat = nullptr;     // [n][4] features of the current sort (collect mode)
    int8_t *pred = nullptr;    // [n] predicted class per sorted position
    float *dx = nullptr;       // dataset features [cap][4]
    int8_t *dy = nullptr;      // dataset classes [cap]
    unsigned long long *dcount = nullptr;
    double *loss = nullptr;    // [2] summed loss, sample count of the last epoch
    int64_t dcap = 0;
    int64_t step = 0;          // Adam step
    int64_t nbuf = 0;          // particles feat / pred can hold
    bool ready = false;        // weights set
    uint32_t keep0 = 0;        // level-0 keep threshold of the collector (of 2^32)
    double keep0_frac = 1.0;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&p);
}

__device__ __forceinline__ uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// B fragment of (W^T)[k0.., n0..] for a row-major weight W[out][in] with row length ld:
// element (k, n) = W[n0 + n][k0 + k].
__device__ __forceinline__ void load_bT(const __nv_bfloat16 *W, int ld, int k0, int n0, uint32_t &b0, uint32_t &b1)
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    const __nv_bfloat16 *row = W + (n0 + g) * ld + k0 + 2 * t;
    b0 = pack_raw(row[0], row[1]);
    b1 = pack_raw(row[8], row[9]);
}

// Features of one particle (FP32), nsg_mlp.cu header.
// x as a float, its significand truncated, built from the double's bits on the integer
// pipe (a conversion instruction would issue to the FP64 pipe, which the step's
// kernels saturate; the features need a few bits only): magnitudes above the float
// range give infinity, below it zero; NaN gives infinity.
__device__ __forceinline__ float f32_trunc(double x)
{
    const unsigned long long u = (unsigned long long)dbits(x);
    const uint32_t sign = (uint32_t)(u >> 63) << 31;
    const int e = (int)((u >> 52) & 0x7ffu) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((uint32_t)e << 23) | (uint32_t)((u >> 29) & 0x7fffffu));
}

// Features of one particle in FP32: log r, v_r over the circular speed, log of ell over
// r times it, log of dt over the local dynamical time r / v_c, with v_c^2 = -gn / r
// from the rank force numerator gn (also in FP32: the features steer only which
// level is tried first, never a result).
// The arithmetic uses the fast hardware forms (approximate logarithm, reciprocal
// square root and division): the features steer, so a few ulp do not matter, and
// training and inference compute them with this same function.
__device__ __forceinline__ void mlp_features(double r, double v, double ell, float gnf, float dtf, float f[4])
{
    const float rf = fmaxf(f32_trunc(r), 1e-30f);
    const float vc2 = fmaxf(__fdividef(-gnf, rf), 1e-30f);
    const float vc = vc2 * rsqrtf(vc2);
    f[0] = __log2f(rf) * 0.125f;
    f[1] = fminf(fmaxf(__fdividef(f32_trunc(v), vc), -8.f), 8.f) * 0.25f;
    f[2] = __log2f(__fdividef(fabsf(f32_trunc(ell)), rf * vc) + 1e-6f) * 0.125f;
    f[3] = __log2f(__fdividef(dtf * vc, rf) + 1e-30f) * 0.125f;
}

// Forward pass of one 16-row tile held by a warp.  x: this thread's rows g and g+8,
// inputs 2t, 2t+1 (only t = 0, 1 carry inputs 0..3).  Writes logits (C layout of
// a 16x8 tile) and, when keep is non-null, the hidden activations as A fragments.
__device__ __forceinline__ void mlp_forward_tile(const __nv_bfloat16 *sW, const float *sB, const float (&xa)[2][2],
                                                 float (&logit)[4], uint32_t (*h1a)[4], uint32_t (*h2a)[4])
{
    const int t = threadIdx.x & 3;
    uint32_t a[4];
    a[0] = pack_bf16(xa[0][0], xa[0][1]);   // row g, inputs 2t, 2t+1
    a[1] = pack_bf16(xa[1][0], xa[1][1]);   // row g+8
    a[2] = 0u;                              // inputs 8..15 are zero
    a[3] = 0u;
    (void)t;
    // layer 1: 16 x 64, bias + relu, as four k-step A fragments of layer 2
    uint32_t h1[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t b0, b1;
        load_bT(sW + kOffW1, kIn, 0, nt * 8, b0, b1);
        mma_bf16(c, a, b0, b1);
        const int col = nt * 8 + 2 * (threadIdx.x & 3);
        const float bb0 = sB[kBB1 + col], bb1 = sB[kBB1 + col + 1];
        const uint32_t lo = pack_bf16(fmaxf(c[0] + bb0, 0.f), fmaxf(c[1] + bb1, 0.f));
        const uint32_t hi = pack_bf16(fmaxf(c[2] + bb0, 0.f), fmaxf(c[3] + bb1, 0.f));
        const int kk = nt >> 1;
        if ((nt & 1) == 0) { h1[kk][0] = lo; h1[kk][1] = hi; }
        else { h1[kk][2] = lo; h1[kk][3] = hi; }
    }
    // layer 2
    uint32_t h2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            uint32_t b0, b1;
            load_bT(sW + kOffW2, kH, kk * 16, nt * 8, b0, b1);
            mma_bf16(c, h1[kk], b0, b1);
        }
        const int col = nt * 8 + 2 * (threadIdx.x & 3);
        const float bb0 = sB[kBB2 + col], bb1 = sB[kBB2 + col + 1];
        const uint32_t lo = pack_bf16(fmaxf(c[0] + bb0, 0.f), fmaxf(c[1] + bb1, 0.f));
        const uint32_t hi = pack_bf16(fmaxf(c[2] + bb0, 0.f), fmaxf(c[3] + bb1, 0.f));
        const int kk = nt >> 1;
        if ((nt & 1) == 0) { h2[kk][0] = lo; h2[kk][1] = hi; }
        else { h2[kk][2] = lo; h2[kk][3] = hi; }
    }
    // layer 3: 16 x 8 logits
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        uint32_t b0, b1;
        load_bT(sW + kOffW3, kH, kk * 16, 0, b0, b1);
        mma_bf16(c, h2[kk], b0, b1);
    }
    const int col = 2 * (threadIdx.x & 3);
    logit[0] = c[0] + sB[kBB3 + col];
    logit[1] = c[1] + sB[kBB3 + col + 1];
    logit[2] = c[2] + sB[kBB3 + col];
    logit[3] = c[3] + sB[kBB3 + col + 1];
    if (h1a) for (int kk = 0; kk < 4; kk++) for (int q = 0; q < 4; q++) h1a[kk][q] = h1[kk][q];
    if (h2a) for (int kk = 0; kk < 4; kk++) for (int q = 0; q < 4; q++) h2a[kk][q] = h2[kk][q];
}

// Loads the bf16 weights and the float biases of the network into shared memory.
__device__ __forceinline__ void mlp_stage(const MlpDev &m, __nv_bfloat16 *sW, float *sB)
{
    for (int k = threadIdx.x; k < kParams; k += blockDim.x) sW[k] = m.wb[k];
    for (int k = threadIdx.x; k < kH; k += blockDim.x) {
        sB[kBB1 + k] = m.w[kOffB1 + k];
        sB[kBB2 + k] = m.w[kOffB2 + k];
    }
    for (int k = threadIdx.x; k < kOut; k += blockDim.x) sB[kBB3 + k] = m.w[kOffB3 + k];
    __syncthreads();
}

// Row-wise argmax of a 16x8 logits tile: returns the class of rows g (lo) and g+8 (hi).
__device__ __forceinline__ void tile_argmax(const float (&lg)[4], int &cls_lo, int &cls_hi)
{
    const int t = threadIdx.x & 3;
    float v0 = lg[0], v1 = lg[2];
    int i0 = 2 * t, i1 = 2 * t;
    if (lg[1] > v0) { v0 = lg[1]; i0 = 2 * t + 1; }
    if (lg[3] > v1) { v1 = lg[3]; i1 = 2 * t + 1; }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
        float w0 = __shfl_xor_sync(0xffffffffu, v0, o), w1 = __shfl_xor_sync(0xffffffffu, v1, o);
        int j0 = __shfl_xor_sync(0xffffffffu, i0, o), j1 = __shfl_xor_sync(0xffffffffu, i1, o);
        if (w0 > v0 || (w0 == v0 && j0 < i0)) { v0 = w0; i0 = j0; }
        if (w1 > v1 || (w1 == v1 && j1 < i1)) { v1 = w1; i1 = j1; }
    }
    cls_lo = i0;
    cls_hi = i1;
}

// Gathers this thread's A-fragment inputs for a tile whose 16 rows are the
// features held by lanes base .. base+15 (f[4] per lane).
__device__ __forceinline__ void tile_inputs(const float (&f)[4], int base, float (&xa)[2][2])
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    // all lanes shuffle every feature; threads with t >= 2 keep zeros
    float v[2][4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        v[0][q] = __shfl_sync(0xffffffffu, f[q], base + g);
        v[1][q] = __shfl_sync(0xffffffffu, f[q], base + g + 8);
    }
    for (int h = 0; h < 2; h++) {
        xa[h][0] = (t == 0) ? v[h][0] : (t == 1) ? v[h][2] : 0.f;
        xa[h][1] = (t == 0) ? v[h][1] : (t == 1) ? v[h][3] : 0.f;
    }
}

struct MlpStepArgs {
    const double *r_src, *v_src, *l_src;
    const unsigned *skip;      // rows below *skip are not read (class 0); null: none
    int64_t n;
    double G, M, dt;
    const DevCounters *ctr;
    Seg seg;
};

// The scheduler's features are those of the state as a step starts, in its array
// order: the previous sort's, so the position of source index i within its halo
// stands for its rank in M(r) = (rank / N) M (exact when nothing crossed since; the
// features only steer which level is tried first).  Feature row of source index i:
__device__ __forceinline__ void state_features(const MlpStepArgs &s, int64_t i, float Gf, float Mf, float Mptf,
                                               float dtf, double r, double v, double ell, float (&f)[4])
{
    const Local L = local_of(s.seg, i, s.n);
    const float gnf = -Gf * ((float)(int32_t)L.i / (float)(int32_t)L.n) * Mf - Gf * Mptf;
    mlp_features(r, v, ell, gnf, dtf, f);
}

// Features of every particle by source index, kept for the training set (collect
// mode).
__global__ void __launch_bounds__(256) k_mlp_features(MlpStepArgs s, MlpDev m)
{
    const float Gf = f32_trunc(s.G), Mf = f32_trunc(s.M), Mptf = f32_trunc(s.ctr->point_mass);
    const float dtf = f32_trunc(s.dt);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < s.n; i += (int64_t)gridDim.x * blockDim.x) {
        float f[4];
        state_features(s, i, Gf, Mf, Mptf, dtf, s.r_src[i], s.v_src[i], s.l_src[i], f);
        *reinterpret_cast<float4 *>(m.feat + i * 4) = make_float4(f[0], f[1], f[2], f[3]);
    }
}

// ------------------------------------------------------------------ inference (tcgen05)
//
// One CTA of 128 threads runs tiles of 128 particles; thread t owns row t of the tile
// (tensor-memory lane t).  Per tile:
//   X [128 x 16] (features, bf16; columns 4..15 zero)       -> shared memory
//   D = X W1^T        (one MMA, M = 128, N = 64, K = 16)     -> tensor memory
//   H = bf16(relu(D + b1))                                   -> shared memory
//   D = H W2^T        (four MMAs, K = 64)                    -> tensor memory
//   H = bf16(relu(D + b2))                                   -> shared memory
//   D = H W3^T        (four MMAs, N = 16: W3's 8 rows and 8 zero rows)
//   logits = D[:, 0..8) + b3, class = first argmax
// One thread issues the MMAs and commits them to an mbarrier that the CTA waits on
// (a bounded wait: on giving up it sets NSG_ST_DEVICE_WAIT).  The weights stay in
// shared memory for the whole launch; the three layers reuse one 64-column
// accumulator, read out before the next layer's MMAs are issued.
constexpr uint32_t kTcRows = 128;                             // particles per tile (MMA M)
constexpr uint32_t kTcN3 = 16;                                // layer-3 N
constexpr uint32_t kTcCols = 64;                              // tensor-memory columns per CTA
constexpr uint32_t kTcW1 = 0;                                 // W1 [64 x 16]
constexpr uint32_t kTcW2 = kTcW1 + kH * kIn * 2;              // W2 [64 x 64]
constexpr uint32_t kTcW3 = kTcW2 + kH * kH * 2;               // W3 [16 x 64]
constexpr uint32_t kTcHid = kTcW3 + kTcN3 * kH * 2;           // H [128 x 64]
// X [128 x 16] is H's first 16 columns (the same layout): it is read by the layer-1
// MMA, which completes before H is written, and rewritten after the layer-3 MMA,
// the last reader of H, completed
constexpr uint32_t kTcX = kTcHid;
constexpr uint32_t kTcBias = kTcHid + kTcRows * kH * 2;       // b1, b2, b3 (FP32)
constexpr uint32_t kTcBar = kTcBias + kBias * 4;              // mbarrier
constexpr uint32_t kTcSlot = kTcBar + 8;                      // tensor-memory address
constexpr uint32_t kTcSmem = kTcSlot + 8;                      // 29 KB: seven CTAs per SM
constexpr uint32_t kTcWaitLimit = 1u << 22;                   // mbarrier polls before giving up
static_assert(kTcBar % 8 == 0 && kTcSlot + 8 <= kTcSmem, "mbarrier alignment, shared-memory size");
// every byte an MMA reads lies inside its operand (last element of each operand)
static_assert(tc_offset(kTcRows, kTcRows - 1, kIn - 1) < kTcRows * kIn * 2, "X layout");
static_assert(tc_offset(kTcRows, kTcRows - 1, kH - 1) < kTcRows * kH * 2, "H layout");
static_assert(tc_offset(kH, kH - 1, kIn - 1) < kH * kIn * 2, "W1 layout");
static_assert(tc_offset(kH, kH - 1, kH - 1) < kH * kH * 2, "W2 layout");
static_assert(tc_offset(kTcN3, kTcN3 - 1, kH - 1) < kTcN3 * kH * 2, "W3 layout");
static_assert(3 * tc_lbo(kTcRows) * 2 + tc_lbo(kTcRows) + 15 * kTcSbo + 128 <= kTcRows * kH * 2, "last H MMA");

// bf16(relu(a + b)) of two columns at once: one paired FP32 addition (IEEE round to
// nearest, as the scalar form), one paired conversion, relu as a paired bf16 maximum
// with zero (rounding is monotone and keeps the sign, so relu after rounding is
// relu before it).
__device__ __forceinline__ uint32_t bias_relu_bf16x2(float a0, float a1, float2 b)
{
    unsigned long long x, y = (unsigned long long)__float_as_uint(b.x) | ((unsigned long long)__float_as_uint(b.y) << 32);
    x = (unsigned long long)__float_as_uint(a0) | ((unsigned long long)__float_as_uint(a1) << 32);
    unsigned long long z;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(x), "l"(y));
    uint32_t p, q;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(p) : "f"(__uint_as_float((uint32_t)(z >> 32))),
        "f"(__uint_as_float((uint32_t)z)));
    asm("max.bf16x2 %0, %1, %2;" : "=r"(q) : "r"(p), "r"(0u));
    return q;
}

// One hidden layer's epilogue for this thread's row: 64 accumulator columns from
// tensor memory, + bias, relu, bf16, into row t of H.
__device__ __forceinline__ void tc_hidden_row(uint32_t trow, const float *__restrict__ bias, unsigned char *hid, int t)
{
    const float4 *b4 = reinterpret_cast<const float4 *>(bias);
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float v[1][16];
        tc_ld16(trow + 16 * c, v[0]);
        tc_wait_ld();
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int k0 = 16 * c + 8 * h;
            const float4 bA = b4[k0 / 4], bB = b4[k0 / 4 + 1];
            const float *a = &v[0][8 * h];
            const uint32_t q0 = bias_relu_bf16x2(a[0], a[1], make_float2(bA.x, bA.y));
            const uint32_t q1 = bias_relu_bf16x2(a[2], a[3], make_float2(bA.z, bA.w));
            const uint32_t q2 = bias_relu_bf16x2(a[4], a[5], make_float2(bB.x, bB.y));
            const uint32_t q3 = bias_relu_bf16x2(a[6], a[7], make_float2(bB.z, bB.w));
            *reinterpret_cast<uint4 *>(hid + tc_offset(kTcRows, t, k0)) = make_uint4(q0, q1, q2, q3);
        }
    }
}

// Completion of the MMAs committed to the barrier: warp 0 polls it (bounded), the
// other warps wait at the CTA barrier that follows.
__device__ __forceinline__ void tc_wait_mma(uint32_t bar, uint32_t &phase, bool &ok, int w)
{
    if (w == 0) ok &= mbar_wait_bounded(bar, phase, kTcWaitLimit);
    __syncthreads();
    phase ^= 1u;
    tc_fence_after();
}

// Predicted class (and, for a feature list, the logits) of every particle.
// FROM_STATE: the features of source index i from the state (state_features), class
// into m.pred[i]; otherwise the features X[i][0..4), class into out[i], logits into
// logits[i][0..8).
template <bool FROM_STATE>
__global__ void __launch_bounds__(kTcRows, 7)
k_mlp_infer_tc(MlpStepArgs s, MlpDev m, const float *__restrict__ X, int64_t cnt, int8_t *__restrict__ out,
               float *__restrict__ logits, unsigned int *status)
{
    extern __shared__ __align__(128) unsigned char tsm[];
    const int t = threadIdx.x, w = t >> 5;
    const uint32_t sb = smem_u32(tsm);
    float *sB = reinterpret_cast<float *>(tsm + kTcBias);
    const uint32_t bar = sb + kTcBar;
    if (w == 0) tc_alloc(sb + kTcSlot, kTcCols);
    // weights into the operand layout, 16 bytes (one row, 8 columns) at a time
    const uint4 *wb = reinterpret_cast<const uint4 *>(m.wb);
    for (int q = t; q < kH * 2; q += kTcRows) {
        const int n = q >> 1, c = q & 1;
        *reinterpret_cast<uint4 *>(tsm + kTcW1 + tc_offset(kH, n, 8 * c)) = wb[(kOffW1 + n * kIn + 8 * c) / 8];
    }
    for (int q = t; q < kH * 8; q += kTcRows) {
        const int n = q >> 3, c = q & 7;
        *reinterpret_cast<uint4 *>(tsm + kTcW2 + tc_offset(kH, n, 8 * c)) = wb[(kOffW2 + n * kH + 8 * c) / 8];
    }
    for (int q = t; q < (int)kTcN3 * 8; q += kTcRows) {
        const int n = q >> 3, c = q & 7;
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(tsm + kTcW3 + tc_offset(kTcN3, n, 8 * c)) =
            n < kOut ? wb[(kOffW3 + n * kH + 8 * c) / 8] : z;
    }
    for (int k = t; k < kH; k += kTcRows) {
        sB[kBB1 + k] = m.w[kOffB1 + k];
        sB[kBB2 + k] = m.w[kOffB2 + k];
    }
    if (t < kOut) sB[kBB3 + t] = m.w[kOffB3 + t];
    if (t == 0) mbar_init(bar, 1u);
    tc_fence_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<const uint32_t *>(tsm + kTcSlot);
    const uint32_t trow = tmem + ((uint32_t)(32 * w) << 16);   // this warp's lanes, column 0
    const uint32_t i64 = tc_idesc_bf16(kTcRows, kH), i16 = tc_idesc_bf16(kTcRows, kTcN3);
    const uint32_t lX = tc_lbo(kTcRows), lW = tc_lbo(kH), lW3 = tc_lbo(kTcN3);

    float Gf = 0.f, Mf = 0.f, Mptf = 0.f, dtf = 0.f;
    if (FROM_STATE) {
        Gf = f32_trunc(s.G); Mf = f32_trunc(s.M); Mptf = f32_trunc(s.ctr->point_mass); dtf = f32_trunc(s.dt);
    }
    const int64_t n = FROM_STATE ? s.n : cnt;
    // rows below `first` belong to the Levi-Civita chains, which may still be writing them
    const int64_t first = (FROM_STATE && s.skip) ? (int64_t)*s.skip : 0;
    uint32_t phase = 0;
    bool ok = true;
    // The inputs of this thread's row of the next tile are loaded while the current
    // tile's MMAs run (issued after layer 1, used at the top of the next tile).
    const float4 *X4 = reinterpret_cast<const float4 *>(X);
    double pr = 0.0, pv = 0.0, pl = 0.0;
    float4 px = make_float4(0.f, 0.f, 0.f, 0.f);
    {
        const int64_t row0 = (int64_t)blockIdx.x * kTcRows + t;
        if (row0 < n && row0 >= first) {
            if (FROM_STATE) { pr = s.r_src[row0]; pv = s.v_src[row0]; pl = s.l_src[row0]; }
            else px = X4[row0];
        }
    }
    for (int64_t tile = blockIdx.x; tile * (int64_t)kTcRows < n; tile += gridDim.x) {
        const int64_t row = tile * (int64_t)kTcRows + t;
        const int64_t nrow = row + (int64_t)gridDim.x * kTcRows;
        float f[4] = {0.f, 0.f, 0.f, 0.f};
        if (row < n && row >= first) {
            if (FROM_STATE) state_features(s, row, Gf, Mf, Mptf, dtf, pr, pv, pl, f);
            else { f[0] = px.x; f[1] = px.y; f[2] = px.z; f[3] = px.w; }
        }
        *reinterpret_cast<uint4 *>(tsm + kTcX + tc_offset(kTcRows, t, 0)) =
            make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), 0u, 0u);
        *reinterpret_cast<uint4 *>(tsm + kTcX + tc_offset(kTcRows, t, 8)) = make_uint4(0u, 0u, 0u, 0u);
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {   // layer 1
            tc_fence_after();
            tc_mma_bf16(tmem, tc_smem_desc(sb + kTcX, lX, kTcSbo), tc_smem_desc(sb + kTcW1, lW, kTcSbo), i64, 0u);
            tc_commit(bar);
        }
        tc_wait_mma(bar, phase, ok, w);
        if (nrow < n && nrow >= first) {
            if (FROM_STATE) { pr = s.r_src[nrow]; pv = s.v_src[nrow]; pl = s.l_src[nrow]; }
            else px = X4[nrow];
        }
        tc_hidden_row(trow, sB + kBB1, tsm + kTcHid, t);
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {   // layer 2
            tc_fence_after();
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                tc_mma_bf16(tmem, tc_smem_desc(sb + kTcHid + 2 * k * lX, lX, kTcSbo),
                            tc_smem_desc(sb + kTcW2 + 2 * k * lW, lW, kTcSbo), i64, k);
            tc_commit(bar);
        }
        tc_wait_mma(bar, phase, ok, w);
        tc_hidden_row(trow, sB + kBB2, tsm + kTcHid, t);
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {   // layer 3
            tc_fence_after();
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                tc_mma_bf16(tmem, tc_smem_desc(sb + kTcHid + 2 * k * lX, lX, kTcSbo),
                            tc_smem_desc(sb + kTcW3 + 2 * k * lW3, lW3, kTcSbo), i16, k);
            tc_commit(bar);
        }
        tc_wait_mma(bar, phase, ok, w);
        float lg[8];
        tc_ld8(trow, lg);
        tc_wait_ld();
        tc_fence_before();   // the next tile's MMAs overwrite these columns after the barrier
        int cls = 0;
        float best = lg[0] + sB[kBB3];
#pragma unroll
        for (int j = 0; j < kOut; j++) {
            lg[j] += sB[kBB3 + j];
            if (j > 0 && lg[j] > best) { best = lg[j]; cls = j; }
        }
        if (row < n) {
            if (FROM_STATE) {
                m.pred[row] = row >= first ? (int8_t)cls : (int8_t)0;
            } else {
                out[row] = (int8_t)cls;
                if (logits) {
                    float4 *lo = reinterpret_cast<float4 *>(logits + row * 8);
                    lo[0] = make_float4(lg[0], lg[1], lg[2], lg[3]);
                    lo[1] = make_float4(lg[4], lg[5], lg[6], lg[7]);
                }
            }
        }
    }
    if (!ok) atomicOr(status, NSG_ST_DEVICE_WAIT);
    __syncthreads();
    tc_fence_after();
    if (w == 0) tc_dealloc(tmem, kTcCols);
}

__device__ __forceinline__ uint32_t hash32(uint64_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
    return (uint32_t)x;
}

// Appends (features, accepted level) of the last step to the training set: every
// particle that needed level >= 1, and level-0 particles with probability keep0.
// Levi-Civita particles are not leapfrog samples and are skipped.
__global__ void __launch_bounds__(256)
k_mlp_append(const int8_t *__restrict__ level, const uint32_t *__restrict__ perm, int64_t n, MlpDev m,
             uint32_t keep0, uint64_t salt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int lv = level[i];
        if (lv >= kLevelLcFallback) continue;
        int cls = (lv < 0) ? kOut - 1 : (lv > kOut - 1 ? kOut - 1 : lv);
        if (cls == 0 && hash32(salt ^ (uint64_t)i) > keep0) continue;
        unsigned long long slot = atomicAdd(m.dcount, 1ull);
        if (slot >= (unsigned long long)m.dcap) continue;
        const uint32_t src = perm[i];   // level of sorted position i, features of its source index
        for (int q = 0; q < 4; q++) m.dx[slot * 4 + q] = m.feat[(int64_t)src * 4 + q];
        m.dy[slot] = (int8_t)cls;
    }
}

// ------------------------------------------------------------------ training

// Generic fragment loads from shared memory for the backward GEMMs.
// A(m, k) = trans ? X[(c0 + k) * ld + r0 + m] : X[(r0 + m) * ld + c0 + k]
__device__ __forceinline__ void load_a_smem(const __nv_bfloat16 *X, int ld, int r0, int c0, bool trans, uint32_t (&a)[4])
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    auto E = [&](int mm, int kk) { return trans ? X[(c0 + kk) * ld + r0 + mm] : X[(r0 + mm) * ld + c0 + kk]; };
    a[0] = pack_raw(E(g, 2 * t), E(g, 2 * t + 1));
    a[1] = pack_raw(E(g + 8, 2 * t), E(g + 8, 2 * t + 1));
    a[2] = pack_raw(E(g, 2 * t + 8), E(g, 2 * t + 9));
    a[3] = pack_raw(E(g + 8, 2 * t + 8), E(g + 8, 2 * t + 9));
}
// B(k, n) = trans ? Y[(n0 + n) * ld + k0 + k] : Y[(k0 + k) * ld + n0 + n]
__device__ __forceinline__ void load_b_smem(const __nv_bfloat16 *Y, int ld, int k0, int n0, bool trans, uint32_t &b0, uint32_t &b1)
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    auto E = [&](int kk, int nn) { return trans ? Y[(n0 + nn) * ld + k0 + kk] : Y[(k0 + kk) * ld + n0 + nn]; };
    b0 = pack_raw(E(2 * t, g), E(2 * t + 1, g));
    b1 = pack_raw(E(2 * t + 8, g), E(2 * t + 9, g));
}

// Stores a 16x8 fp32 C tile (rows r0.., cols c0..) into a bf16 row-major matrix.
__device__ __forceinline__ void store_c_bf16(__nv_bfloat16 *Y, int ld, int r0, int c0, const float (&c)[4])
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    Y[(r0 + g) * ld + c0 + 2 * t] = __float2bfloat16_rn(c[0]);
    Y[(r0 + g) * ld + c0 + 2 * t + 1] = __float2bfloat16_rn(c[1]);
    Y[(r0 + g + 8) * ld + c0 + 2 * t] = __float2bfloat16_rn(c[2]);
    Y[(r0 + g + 8) * ld + c0 + 2 * t + 1] = __float2bfloat16_rn(c[3]);
}

// Accumulates a 16x8 fp32 C tile into a float row-major matrix in shared memory.
__device__ __forceinline__ void accum_c(float *Y, int ld, int r0, int c0, const float (&c)[4])
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    atomicAdd(&Y[(r0 + g) * ld + c0 + 2 * t], c[0]);
    atomicAdd(&Y[(r0 + g) * ld + c0 + 2 * t + 1], c[1]);
    atomicAdd(&Y[(r0 + g + 8) * ld + c0 + 2 * t], c[2]);
    atomicAdd(&Y[(r0 + g + 8) * ld + c0 + 2 * t + 1], c[3]);
}

constexpr int kTrainWarps = 4;   // one 16-sample tile per warp

// Forward + backward of softmax cross-entropy over samples [begin, end) of the
// dataset; sample weights w_c per class; gradients summed (FP32) into m.g, loss
// summed into m.loss.  Each block loops over tiles of 16 samples per warp and
// reduces its gradients in shared memory before one global add per parameter.
__global__ void __launch_bounds__(kTrainWarps * 32)
k_mlp_train(MlpDev m, const float *__restrict__ X, const int8_t *__restrict__ Y, const int32_t *__restrict__ order,
            int64_t begin, int64_t end, const float *__restrict__ cls_w)
{
    __shared__ __nv_bfloat16 sW[kParams];
    __shared__ float sB[kBias];
    __shared__ float sLoss;
    // dynamic shared memory: gradient accumulator, then per-warp activation tiles
    extern __shared__ __align__(16) unsigned char dsm[];
    float *sG = reinterpret_cast<float *>(dsm);
    typedef __nv_bfloat16 TileX[16 * kIn];
    typedef __nv_bfloat16 TileH[16 * kH];
    typedef __nv_bfloat16 Tile16[16 * 16];
    TileX *sX = reinterpret_cast<TileX *>(sG + kParams);
    TileH *sH1 = reinterpret_cast<TileH *>(sX + kTrainWarps);
    TileH *sH2 = sH1 + kTrainWarps;
    TileH *sD = sH2 + kTrainWarps;                    // dZ (reused per layer)
    Tile16 *sD3 = reinterpret_cast<Tile16 *>(sD + kTrainWarps);   // dZ3 padded to 16 columns
    mlp_stage(m, sW, sB);
    for (int k = threadIdx.x; k < kParams; k += blockDim.x) sG[k] = 0.f;
    if (threadIdx.x == 0) sLoss = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int64_t ntile = (end - begin + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * kTrainWarps + w; tile < ntile;
         tile += (int64_t)gridDim.x * kTrainWarps) {
        const int64_t s0 = begin + tile * 16;
        // load features: lanes 0..15 one sample each
        float f[4] = {0.f, 0.f, 0.f, 0.f};
        int label = -1;
        float wgt = 0.f;
        if (lane < 16 && s0 + lane < end) {
            const int64_t idx = order ? order[s0 + lane] : s0 + lane;
            for (int q = 0; q < 4; q++) f[q] = X[idx * 4 + q];
            label = Y[idx];
            wgt = cls_w[label];
        }
        // X tile [16 samples][16 inputs]: entry q = lane + 32 j has row 2j + lane/16
        // and column lane % 16; every lane takes part in every shuffle
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int row = 2 * j + (lane >> 4), col = lane & 15;
            const float v0 = __shfl_sync(0xffffffffu, f[0], row), v1 = __shfl_sync(0xffffffffu, f[1], row);
            const float v2 = __shfl_sync(0xffffffffu, f[2], row), v3 = __shfl_sync(0xffffffffu, f[3], row);
            const float val = col == 0 ? v0 : col == 1 ? v1 : col == 2 ? v2 : col == 3 ? v3 : 0.f;
            sX[w][row * kIn + col] = __float2bfloat16_rn(val);
        }
        float xa[2][2];
        tile_inputs(f, 0, xa);
        float lg[4];
        uint32_t h1[4][4], h2[4][4];
        mlp_forward_tile(sW, sB, xa, lg, h1, h2);
        // hidden activations to shared memory (row-major [sample][unit])
        for (int kk = 0; kk < 4; kk++) {
            __nv_bfloat162 *p;
            const int c0 = kk * 16 + 2 * t;
            p = reinterpret_cast<__nv_bfloat162 *>(&sH1[w][g * kH + c0]);          *p = *reinterpret_cast<__nv_bfloat162 *>(&h1[kk][0]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH1[w][(g + 8) * kH + c0]);    *p = *reinterpret_cast<__nv_bfloat162 *>(&h1[kk][1]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH1[w][g * kH + c0 + 8]);      *p = *reinterpret_cast<__nv_bfloat162 *>(&h1[kk][2]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH1[w][(g + 8) * kH + c0 + 8]);*p = *reinterpret_cast<__nv_bfloat162 *>(&h1[kk][3]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH2[w][g * kH + c0]);          *p = *reinterpret_cast<__nv_bfloat162 *>(&h2[kk][0]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH2[w][(g + 8) * kH + c0]);    *p = *reinterpret_cast<__nv_bfloat162 *>(&h2[kk][1]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH2[w][g * kH + c0 + 8]);      *p = *reinterpret_cast<__nv_bfloat162 *>(&h2[kk][2]);
            p = reinterpret_cast<__nv_bfloat162 *>(&sH2[w][(g + 8) * kH + c0 + 8]);*p = *reinterpret_cast<__nv_bfloat162 *>(&h2[kk][3]);
        }
        // softmax cross-entropy: dZ3 = w (softmax - onehot); rows g (lg[0..1]) and g+8 (lg[2..3])
        const int lab0 = __shfl_sync(0xffffffffu, label, g), lab1 = __shfl_sync(0xffffffffu, label, g + 8);
        const float wg0 = __shfl_sync(0xffffffffu, wgt, g), wg1 = __shfl_sync(0xffffffffu, wgt, g + 8);
        float mx0 = fmaxf(lg[0], lg[1]), mx1 = fmaxf(lg[2], lg[3]);
        for (int o = 1; o <= 2; o <<= 1) {
            mx0 = fmaxf(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
            mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        }
        float e[4] = {__expf(lg[0] - mx0), __expf(lg[1] - mx0), __expf(lg[2] - mx1), __expf(lg[3] - mx1)};
        float s0s = e[0] + e[1], s1s = e[2] + e[3];
        for (int o = 1; o <= 2; o <<= 1) {
            s0s += __shfl_xor_sync(0xffffffffu, s0s, o);
            s1s += __shfl_xor_sync(0xffffffffu, s1s, o);
        }
        float dz[4];
        const int col = 2 * t;
        for (int q = 0; q < 4; q++) {
            const int row_hi = q >> 1, cc = col + (q & 1);
            const int lab = row_hi ? lab1 : lab0;
            const float wg = row_hi ? wg1 : wg0;
            const float p = e[q] / (row_hi ? s1s : s0s);
            dz[q] = (lab >= 0) ? wg * (p - (cc == lab ? 1.f : 0.f)) : 0.f;
            if (lab >= 0 && cc == lab) atomicAdd(&sLoss, -wg * logf(fmaxf(p, 1e-30f)));
        }
        // dZ3 into shared memory, padded to 16 columns with zeros
        for (int q = lane; q < 16 * 16; q += 32) sD3[w][q] = __float2bfloat16_rn(0.f);
        __syncwarp();
        {
            float c[4] = {dz[0], dz[1], dz[2], dz[3]};
            store_c_bf16(sD3[w], 16, 0, 0, c);
            // bias gradient b3
            atomicAdd(&sG[kOffB3 + col], dz[0] + dz[2]);
            atomicAdd(&sG[kOffB3 + col + 1], dz[1] + dz[3]);
        }
        __syncwarp();
        // dW3^T [64 x 8] = H2^T (64 x 16) . dZ3 (16 x 8)
        for (int mt = 0; mt < 4; mt++) {
            uint32_t a[4], b0, b1;
            load_a_smem(sH2[w], kH, mt * 16, 0, true, a);
            load_b_smem(sD3[w], 16, 0, 0, false, b0, b1);
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16(c, a, b0, b1);
            // c(m = hidden unit, n = class) -> dW3[class][unit]
            atomicAdd(&sG[kOffW3 + (2 * t) * kH + mt * 16 + g], c[0]);
            atomicAdd(&sG[kOffW3 + (2 * t + 1) * kH + mt * 16 + g], c[1]);
            atomicAdd(&sG[kOffW3 + (2 * t) * kH + mt * 16 + g + 8], c[2]);
            atomicAdd(&sG[kOffW3 + (2 * t + 1) * kH + mt * 16 + g + 8], c[3]);
        }
        // dH2 [16 x 64] = dZ3 (16 x 16 padded) . W3 (16 x 64, rows 8..15 unused -> zero A columns)
        for (int nt = 0; nt < 8; nt++) {
            uint32_t a[4], b0, b1;
            load_a_smem(sD3[w], 16, 0, 0, false, a);
            // B(k, n) = W3[k][n] for k < 8; zero for k >= 8 (A is zero there too)
            const __nv_bfloat16 *W3 = sW + kOffW3;
            b0 = pack_raw(W3[(2 * t) * kH + nt * 8 + g], W3[(2 * t + 1) * kH + nt * 8 + g]);
            b1 = 0u;
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16(c, a, b0, b1);
            // relu'(H2): H2 > 0
            const int cc = nt * 8 + 2 * t;
            float h00 = __bfloat162float(sH2[w][g * kH + cc]), h01 = __bfloat162float(sH2[w][g * kH + cc + 1]);
            float h10 = __bfloat162float(sH2[w][(g + 8) * kH + cc]), h11 = __bfloat162float(sH2[w][(g + 8) * kH + cc + 1]);
            c[0] = h00 > 0.f ? c[0] : 0.f; c[1] = h01 > 0.f ? c[1] : 0.f;
            c[2] = h10 > 0.f ? c[2] : 0.f; c[3] = h11 > 0.f ? c[3] : 0.f;
            atomicAdd(&sG[kOffB2 + cc], c[0] + c[2]);
            atomicAdd(&sG[kOffB2 + cc + 1], c[1] + c[3]);
            store_c_bf16(sD[w], kH, 0, nt * 8, c);   // dZ2
        }
        __syncwarp();
        // dW2 [64 x 64] = dZ2^T (64 x 16) . H1 (16 x 64)
        for (int mt = 0; mt < 4; mt++)
            for (int nt = 0; nt < 8; nt++) {
                uint32_t a[4], b0, b1;
                load_a_smem(sD[w], kH, mt * 16, 0, true, a);
                load_b_smem(sH1[w], kH, 0, nt * 8, false, b0, b1);
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                mma_bf16(c, a, b0, b1);
                accum_c(sG + kOffW2, kH, mt * 16, nt * 8, c);
            }
        // dH1 [16 x 64] = dZ2 (16 x 64) . W2 (64 x 64);  B(k, n) = W2[k][n]
        float dh1[8][4];
        for (int nt = 0; nt < 8; nt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            for (int kk = 0; kk < 4; kk++) {
                uint32_t a[4], b0, b1;
                load_a_smem(sD[w], kH, 0, kk * 16, false, a);
                load_b_smem(sW + kOffW2, kH, kk * 16, nt * 8, false, b0, b1);
                mma_bf16(c, a, b0, b1);
            }
            const int cc = nt * 8 + 2 * t;
            float h00 = __bfloat162float(sH1[w][g * kH + cc]), h01 = __bfloat162float(sH1[w][g * kH + cc + 1]);
            float h10 = __bfloat162float(sH1[w][(g + 8) * kH + cc]), h11 = __bfloat162float(sH1[w][(g + 8) * kH + cc + 1]);
            dh1[nt][0] = h00 > 0.f ? c[0] : 0.f; dh1[nt][1] = h01 > 0.f ? c[1] : 0.f;
            dh1[nt][2] = h10 > 0.f ? c[2] : 0.f; dh1[nt][3] = h11 > 0.f ? c[3] : 0.f;
        }
        __syncwarp();
        for (int nt = 0; nt < 8; nt++) {
            const int cc = nt * 8 + 2 * t;
            atomicAdd(&sG[kOffB1 + cc], dh1[nt][0] + dh1[nt][2]);
            atomicAdd(&sG[kOffB1 + cc + 1], dh1[nt][1] + dh1[nt][3]);
            store_c_bf16(sD[w], kH, 0, nt * 8, dh1[nt]);   // dZ1
        }
        __syncwarp();
        // dW1 [64 x 16] = dZ1^T (64 x 16) . X (16 x 16)
        for (int mt = 0; mt < 4; mt++)
            for (int nt = 0; nt < 2; nt++) {
                uint32_t a[4], b0, b1;
                load_a_smem(sD[w], kH, mt * 16, 0, true, a);
                load_b_smem(sX[w], kIn, 0, nt * 8, false, b0, b1);
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                mma_bf16(c, a, b0, b1);
                accum_c(sG + kOffW1, kIn, mt * 16, nt * 8, c);
            }
        __syncwarp();
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kParams; k += blockDim.x)
        if (sG[k] != 0.f) atomicAdd(&m.g[k], sG[k]);
    if (threadIdx.x == 0) atomicAdd(&m.loss[0], (double)sLoss);
}

// Adam step on the master weights (gradients divided by the batch weight), then
// the bf16 copies; clears the gradient.  Input columns 4..15 of W1 stay zero.
__global__ void k_mlp_adam(MlpDev m, float lr, float inv_batch, float b1c, float b2c)
{
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kParams; k += gridDim.x * blockDim.x) {
        float gk = m.g[k] * inv_batch;
        if (k < kW1 && (k % kIn) >= 4) gk = 0.f;
        const float mk = beta1 * m.m[k] + (1.f - beta1) * gk;
        const float vk = beta2 * m.v[k] + (1.f - beta2) * gk * gk;
        m.m[k] = mk;
        m.v[k] = vk;
        float wk = m.w[k] - lr * (mk / b1c) / (sqrtf(vk / b2c) + eps);
        if (k < kW1 && (k % kIn) >= 4) wk = 0.f;
        m.w[k] = wk;
        m.wb[k] = __float2bfloat16_rn(wk);
        m.g[k] = 0.f;
    }
}

__global__ void k_mlp_refresh_bf16(MlpDev m)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kParams; k += gridDim.x * blockDim.x)
        m.wb[k] = __float2bfloat16_rn(m.w[k]);
}

}  // namespace nsg

namespace nsg {

size_t mlp_train_smem()
{
    return (size_t)kParams * sizeof(float) +
           (size_t)kTrainWarps * (16 * kIn + 3 * 16 * kH + 16 * 16) * sizeof(__nv_bfloat16);
}

}  // namespace nsg

// ------------------------------------------------------------------ host side

namespace nsg {

static int mlp_alloc(nsg_ctx *c)
{
    if (c->mlp) return NSG_OK;
    MlpDev *m = new MlpDev();
    cudaError_t e = cudaMalloc((void **)&m->w, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->g, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->m, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->v, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->wb, kParams * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->dcount, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->loss, 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(m->g, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->m, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->v, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->dcount, 0, sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_train_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_infer_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_infer_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    c->mlp = m;
    if (e != cudaSuccess) return cuda_err(c, e, "mlp allocation");
    return NSG_OK;
}

void mlp_free(nsg_ctx *c)
{
    MlpDev *m = c->mlp;
    if (!m) return;
    cudaFree(m->w); cudaFree(m->g); cudaFree(m->m); cudaFree(m->v); cudaFree(m->wb);
    cudaFree(m->dcount); cudaFree(m->loss); cudaFree(m->feat); cudaFree(m->pred);
    cudaFree(m->dx); cudaFree(m->dy);
    delete m;
    c->mlp = nullptr;
}

static int mlp_ensure_n(nsg_ctx *c)
{
    MlpDev *m = c->mlp;
    if (m->nbuf >= c->n) return NSG_OK;
    cudaFree(m->feat); cudaFree(m->pred);
    m->feat = nullptr; m->pred = nullptr;
    cudaError_t e = cudaMalloc((void **)&m->feat, (size_t)c->n * 4 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->pred, (size_t)c->n);
    if (e != cudaSuccess) return cuda_err(c, e, "mlp buffers");
    m->nbuf = c->n;
    return NSG_OK;
}

static MlpStepArgs step_args(nsg_ctx *c, int src = -1)
{
    MlpStepArgs s;
    if (src < 0) src = c->cur;
    s.r_src = c->r[src]; s.v_src = c->vr[src]; s.l_src = c->ell[src];
    s.skip = nullptr;
    s.n = c->n; s.G = c->p.G; s.M = c->p.M_total; s.dt = c->p.dt;
    s.ctr = c->ctr;
    s.seg = seg_table(c);
    return s;
}

// CTAs of the inference kernel: one tile of 128 particles at a time, at most seven
// per SM (29 KB of shared memory each; 64 of the SM's 512 tensor-memory columns).
static int infer_grid(const nsg_ctx *c, int64_t n)
{
    const int64_t tiles = (n + kTcRows - 1) / kTcRows;
    const int64_t cap = (int64_t)c->num_sms * 7;
    return (int)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

// Predicted class per source index of the state as the step starts (copy c->cur).
int mlp_predict_state(nsg_ctx *c, const int8_t **pred, cudaStream_t st, int buf, const unsigned *skip)
{
    if (!c->mlp || !c->mlp->ready) return set_err(c, NSG_ESTATE, "learned schedule needs nsg_mlp_init or trained weights");
    if (int rc = mlp_ensure_n(c)) return rc;
    ProfScope ps(c, "mlp_predict", (double)c->n * (4 + 28 + 1), st);
    MlpStepArgs sa = step_args(c, buf);
    sa.skip = skip;
    k_mlp_infer_tc<true><<<infer_grid(c, c->n), kTcRows, kTcSmem, st>>>(sa, *c->mlp, nullptr, 0, nullptr, nullptr,
                                                                         &c->ctr->status);
    c->launches += 1;
    *pred = c->mlp->pred;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp predict");
}

const int8_t *mlp_pred_buffer(nsg_ctx *c) { return c->mlp ? c->mlp->pred : nullptr; }

// Features of the state as the step starts, kept for the training set (collect mode).
int mlp_features_state(nsg_ctx *c, cudaStream_t st)
{
    if (int rc = mlp_ensure_n(c)) return rc;
    k_mlp_features<<<grid_for(c, c->n, 256, 4), 256, 0, st>>>(step_args(c), *c->mlp);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp features");
}

int mlp_append_levels(nsg_ctx *c)
{
    MlpDev *m = c->mlp;
    k_mlp_append<<<grid_for(c, c->n, 256, 4), 256, 0, c->stream>>>(c->level, c->perm, c->n, *m, m->keep0,
                                                                  0x9E3779B97F4A7C15ull * (uint64_t)(c->steps_done + 1));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp append");
}

}  // namespace nsg

using namespace nsg;

extern "C" {

// The network's buffers are also read and written by kernels on the context's
// streams (collection, learned steps); the calls below touch them with
// synchronous copies and launches on the default stream, so they first wait for
// the context's streams to finish.
static void mlp_quiesce(nsg_ctx *c)
{
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
}

int nsg_mlp_num_params(void) { return kParams; }

int nsg_mlp_init(nsg_ctx *c, uint64_t seed)
{
    if (c) c->pred_epoch = -1;   // new weights: the predictions made so far are stale
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    mlp_quiesce(c);
    if (int rc = mlp_alloc(c)) return rc;
    // He-uniform initial weights from a seeded generator; zero biases and padding
    std::vector<float> w(kParams, 0.f);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
    auto uni = [&]() {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        return (float)((s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    for (int o = 0; o < kH; o++) for (int i = 0; i < 4; i++) w[kOffW1 + o * kIn + i] = uni() * sqrtf(6.f / 4.f);
    for (int k = 0; k < kW2; k++) w[kOffW2 + k] = uni() * sqrtf(6.f / kH);
    for (int k = 0; k < kW3; k++) w[kOffW3 + k] = uni() * sqrtf(6.f / kH);
    return nsg_mlp_set_weights(c, w.data(), kParams);
}

int nsg_mlp_set_weights(nsg_ctx *c, const float *w, int64_t count)
{
    if (c) c->pred_epoch = -1;   // new weights: the predictions made so far are stale
    if (!c || !w || count != kParams) return set_err(c, NSG_EINVAL, "weights must have nsg_mlp_num_params() floats");
    mlp_quiesce(c);
    if (int rc = mlp_alloc(c)) return rc;
    MlpDev *m = c->mlp;
    cudaError_t e = cudaMemcpy(m->w, w, kParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_mlp_refresh_bf16<<<8, 256>>>(*m);
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) return cuda_err(c, e, "set weights");
    m->ready = true;
    m->step = 0;
    cudaMemset(m->m, 0, kParams * sizeof(float));
    cudaMemset(m->v, 0, kParams * sizeof(float));
    return NSG_OK;
}

int nsg_mlp_get_weights(nsg_ctx *c, float *w, int64_t count)
{
    if (!c || !w || count != kParams) return set_err(c, NSG_EINVAL, "weights must have nsg_mlp_num_params() floats");
    if (!c->mlp) return set_err(c, NSG_ESTATE, "no network");
    mlp_quiesce(c);
    cudaError_t e = cudaMemcpy(w, c->mlp->w, kParams * sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "get weights");
}

int nsg_mlp_collect(nsg_ctx *c, int nsteps, double keep_level0, int64_t capacity)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (nsteps < 0 || capacity <= 0 || !(keep_level0 >= 0.0 && keep_level0 <= 1.0))
        return set_err(c, NSG_EINVAL, "bad collect arguments");
    if (c->p.method == NSG_METHOD_KDK) return set_err(c, NSG_EINVAL, "levels exist only for the adaptive methods");
    mlp_quiesce(c);
    if (int rc = mlp_alloc(c)) return rc;
    MlpDev *m = c->mlp;
    if (m->dcap != capacity) {
        cudaFree(m->dx); cudaFree(m->dy);
        m->dx = nullptr; m->dy = nullptr; m->dcap = 0;
        cudaError_t e = cudaMalloc((void **)&m->dx, (size_t)capacity * 4 * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->dy, (size_t)capacity);
        if (e == cudaSuccess) e = cudaMemset(m->dcount, 0, sizeof(unsigned long long));
        if (e != cudaSuccess) return cuda_err(c, e, "dataset allocation");
        m->dcap = capacity;
    }
    m->keep0 = (uint32_t)(keep_level0 * 4294967295.0);
    m->keep0_frac = keep_level0;
    const int32_t sched = c->p.sched;
    c->p.sched = NSG_SCHED_PLAIN;   // levels of the plain method are the labels
    c->mlp_collect = true;
    int rc = nsg_step(c, nsteps);
    c->mlp_collect = false;
    c->p.sched = sched;
    return rc;
}

int nsg_mlp_dataset(nsg_ctx *c, int64_t *count, float *X, int8_t *y, int64_t max)
{
    if (!c || !count) return set_err(c, NSG_EINVAL, "null argument");
    if (!c->mlp || !c->mlp->dx) { *count = 0; return NSG_OK; }
    mlp_quiesce(c);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, c->mlp->dcount, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(c, e, "dataset count");
    int64_t n = (int64_t)(h < (unsigned long long)c->mlp->dcap ? h : (unsigned long long)c->mlp->dcap);
    *count = n;
    int64_t k = n < max ? n : max;
    if (X && k > 0) e = cudaMemcpy(X, c->mlp->dx, (size_t)k * 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && y && k > 0) e = cudaMemcpy(y, c->mlp->dy, (size_t)k, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "dataset read");
}

// One pass of forward + backward over samples [0, nb) with class weights cls_w[8];
// gradients (summed, not averaged) land in m->g, the summed loss in m->loss[0].
static int mlp_grad_pass(nsg_ctx *c, const float *d_X, const int8_t *d_y, const int32_t *d_order, int64_t begin,
                         int64_t end, const float *d_w)
{
    MlpDev *m = c->mlp;
    const int64_t tiles = (end - begin + 15) / 16;
    int blocks = (int)((tiles + kTrainWarps - 1) / kTrainWarps);
    if (blocks > c->num_sms * 4) blocks = c->num_sms * 4;
    if (blocks < 1) blocks = 1;
    k_mlp_train<<<blocks, kTrainWarps * 32, mlp_train_smem(), c->stream>>>(*m, d_X, d_y, d_order, begin, end, d_w);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp train kernel");
}

int nsg_mlp_grad(nsg_ctx *c, const float *X, const int8_t *y, int64_t nb, const float *cls_w, float *grad,
                 double *loss)
{
    if (!c || !X || !y || nb <= 0 || !cls_w) return set_err(c, NSG_EINVAL, "bad gradient arguments");
    if (!c->mlp || !c->mlp->ready) return set_err(c, NSG_ESTATE, "no network");
    mlp_quiesce(c);
    for (int64_t k = 0; k < nb; k++)
        if (y[k] < 0 || y[k] >= kOut) return set_err(c, NSG_EINVAL, "class labels must be in 0..7");
    MlpDev *m = c->mlp;
    float *d_X = nullptr, *d_w = nullptr;
    int8_t *d_y = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_X, (size_t)nb * 16);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_y, (size_t)nb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_w, 8 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(d_X, X, (size_t)nb * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_y, y, (size_t)nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_w, cls_w, 8 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->g, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->loss, 0, 2 * sizeof(double));
    int rc = NSG_OK;
    if (e == cudaSuccess) rc = mlp_grad_pass(c, d_X, d_y, nullptr, 0, nb, d_w);
    if (e == cudaSuccess && rc == NSG_OK) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && rc == NSG_OK && grad) e = cudaMemcpy(grad, m->g, kParams * sizeof(float), cudaMemcpyDeviceToHost);
    double hl[2] = {0, 0};
    if (e == cudaSuccess && rc == NSG_OK) e = cudaMemcpy(hl, m->loss, sizeof(hl), cudaMemcpyDeviceToHost);
    if (loss) *loss = hl[0];
    cudaMemset(m->g, 0, kParams * sizeof(float));
    cudaFree(d_X); cudaFree(d_y); cudaFree(d_w);
    if (rc) return rc;
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp grad");
}

int nsg_mlp_train(nsg_ctx *c, int epochs, int batch, float lr, uint64_t seed, double *final_loss)
{
    if (c) c->pred_epoch = -1;   // new weights: the predictions made so far are stale
    if (!c || epochs < 0 || batch < 16 || !(lr > 0.f)) return set_err(c, NSG_EINVAL, "bad training arguments");
    if (!c->mlp || !c->mlp->ready) return set_err(c, NSG_ESTATE, "call nsg_mlp_init first");
    mlp_quiesce(c);
    MlpDev *m = c->mlp;
    int64_t n = 0;
    if (int rc = nsg_mlp_dataset(c, &n, nullptr, nullptr, 0)) return rc;
    if (n <= 0) return set_err(c, NSG_ESTATE, "empty training set: call nsg_mlp_collect first");
    // class weights restore the true prior of level 0 (subsampled by keep0)
    float hw[8];
    for (int k = 0; k < 8; k++) hw[k] = 1.f;
    hw[0] = (float)(m->keep0_frac > 0 ? 1.0 / m->keep0_frac : 1.0);
    std::vector<int8_t> hy((size_t)n);
    cudaError_t e = cudaMemcpy(hy.data(), m->dy, (size_t)n, cudaMemcpyDeviceToHost);
    std::vector<int32_t> order((size_t)n);
    for (int64_t k = 0; k < n; k++) order[k] = (int32_t)k;
    int32_t *d_order = nullptr;
    float *d_w = nullptr;
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_order, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_w, 8 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(d_w, hw, sizeof(hw), cudaMemcpyHostToDevice);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 7;
    double last = 0.0;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
        for (int64_t k = n - 1; k > 0; k--) {      // Fisher-Yates shuffle
            s ^= s << 13; s ^= s >> 7; s ^= s << 17;
            int64_t j = (int64_t)(s % (uint64_t)(k + 1));
            std::swap(order[k], order[j]);
        }
        e = cudaMemcpyAsync(d_order, order.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, 2 * sizeof(double), c->stream);
        double wsum_epoch = 0.0;
        for (int64_t b0 = 0; b0 < n && e == cudaSuccess; b0 += batch) {
            const int64_t b1 = b0 + batch < n ? b0 + batch : n;
            double wsum = 0.0;
            for (int64_t k = b0; k < b1; k++) wsum += hw[hy[order[k]]];
            wsum_epoch += wsum;
            if (int rc = mlp_grad_pass(c, m->dx, m->dy, d_order, b0, b1, d_w)) { cudaFree(d_order); cudaFree(d_w); return rc; }
            m->step++;
            const float b1c = 1.f - powf(0.9f, (float)m->step), b2c = 1.f - powf(0.999f, (float)m->step);
            k_mlp_adam<<<8, 256, 0, c->stream>>>(*m, lr, (float)(1.0 / wsum), b1c, b2c);
            e = cudaGetLastError();
        }
        double hl[2] = {0, 0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(hl, m->loss, sizeof(hl), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        last = hl[0] / (wsum_epoch > 0 ? wsum_epoch : 1.0);
    }
    cudaFree(d_order);
    cudaFree(d_w);
    if (final_loss) *final_loss = last;
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp train");
}

int nsg_mlp_predict(nsg_ctx *c, const float *X, int64_t nb, int8_t *cls, float *logits)
{
    if (!c || !X || nb <= 0 || !cls) return set_err(c, NSG_EINVAL, "bad predict arguments");
    if (!c->mlp || !c->mlp->ready) return set_err(c, NSG_ESTATE, "no network");
    mlp_quiesce(c);
    float *d_X = nullptr, *d_l = nullptr;
    int8_t *d_c = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_X, (size_t)nb * 16);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_c, (size_t)nb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_l, (size_t)nb * 32);
    if (e == cudaSuccess) e = cudaMemcpy(d_X, X, (size_t)nb * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_mlp_infer_tc<false><<<infer_grid(c, nb), kTcRows, kTcSmem, c->stream>>>(MlpStepArgs{}, *c->mlp, d_X, nb, d_c,
                                                                                   d_l, &c->ctr->status);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpy(cls, d_c, (size_t)nb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && logits) e = cudaMemcpy(logits, d_l, (size_t)nb * 32, cudaMemcpyDeviceToHost);
    cudaFree(d_X); cudaFree(d_c); cudaFree(d_l);
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "mlp predict");
}

}  // extern "C"
