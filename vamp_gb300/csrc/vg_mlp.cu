// Tensor-core (tcgen05) kernels of the learned block ordering: a BF16 GEMM with FP32 TMEM
// accumulation and fused epilogues, the building block of the MLP's forward and backward passes.
#include "../../include/vamp_gb300.h"
#include "vg_internal.h"
#include "vg_tc.cuh"

#include <cuda_bf16.h>

#include <string>

namespace vg
{
    constexpr int kGemmKC = 128;          // K columns staged per chunk
    constexpr uint32_t kWaitLimit = 1u << 22;

    enum GemmEpilogue : int
    {
        kEpiStoreF32 = 0,      // D (fp32)
        kEpiBiasReluBf16 = 1,  // relu(D + bias) as bf16
    };

    struct GemmParams
    {
        const __nv_bfloat16 *a;  // [M][K]
        const __nv_bfloat16 *b;  // [N][K]
        float *d_f32;            // [M][N]
        __nv_bfloat16 *d_bf16;   // [M][N]
        const float *bias;       // [N]
        int M, N, K;
        int *err;                // set to 1 if a wait gave up
        // polls of an MMA-completion barrier before the kernel gives up (the wait for MMAs still
        // in flight before the tensor memory is released always uses kWaitLimit)
        uint32_t wait_limit = kWaitLimit;
    };

    // D[M x N] = A[M x K] B[N x K]^T.  One CTA of 128 threads per 128-row tile; N in 16..256 (a
    // multiple of 16), K a multiple of 16, M a multiple of 128.  Operands are staged in K chunks
    // into shared memory (core-matrix layout, vg_tc.cuh), one thread issues the MMAs, the
    // accumulator lives in TMEM and each warp reads back its 32 rows.
    template <int EPI>
    __global__ void __launch_bounds__(128, 1) gemm_bf16_kernel(const GemmParams p)
    {
        extern __shared__ __align__(1024) unsigned char gemm_smem[];
        __shared__ uint64_t bar;
        __shared__ uint32_t tmem_slot;
        unsigned char *sa = gemm_smem;  // 128 x KC
        unsigned char *sb = gemm_smem + 128 * kGemmKC * 2;  // N x KC
        const int tid = threadIdx.x;
        const int warp = tid >> 5;
        const int m0 = blockIdx.x * 128;
        const uint32_t tcols = p.N <= 32 ? 32u : (p.N <= 64 ? 64u : (p.N <= 128 ? 128u : 256u));
        __shared__ int skip;

        // after an earlier kernel gave up, do nothing (decided once per CTA, so all threads agree)
        if (tid == 0)
            skip = *static_cast<volatile int *>(p.err);
        __syncthreads();
        if (skip)
            return;
        if (warp == 0)
        {
            tc::tmem_alloc(&tmem_slot, tcols);
        }
        if (tid == 0)
        {
            tc::mbar_init(&bar, 1);
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tmem = tmem_slot;
        const uint32_t idesc = tc::idesc_bf16_f32(128, p.N);
        bool ok = true;
        uint32_t phase = 0;

        for (int k0 = 0; k0 < p.K; k0 += kGemmKC)
        {
            const int kc = min(kGemmKC, p.K - k0);
            const int units = kc >> 3;  // 16-byte units per row in this chunk
            // stage A rows m0..m0+127 and B rows 0..N-1 (16-byte units, K-contiguous in global)
            for (int u = tid; u < 128 * units; u += 128)
            {
                const int r = u / units, g = u % units;
                const uint4 v = *reinterpret_cast<const uint4 *>(p.a + static_cast<size_t>(m0 + r) * p.K + k0 + 8 * g);
                *reinterpret_cast<uint4 *>(sa + tc::tile_offset(r, 8 * g, kGemmKC)) = v;
            }
            for (int u = tid; u < p.N * units; u += 128)
            {
                const int r = u / units, g = u % units;
                const uint4 v = *reinterpret_cast<const uint4 *>(p.b + static_cast<size_t>(r) * p.K + k0 + 8 * g);
                *reinterpret_cast<uint4 *>(sb + tc::tile_offset(r, 8 * g, kGemmKC)) = v;
            }
            tc::fence_smem_to_async();
            __syncthreads();
            if (tid == 0)
            {
                tc::fence_after_sync();
                const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
                constexpr uint32_t lbo = 128, sbo = (kGemmKC / 8) * 128;
                for (int kk = 0; kk < kc / 16; ++kk)
                {
                    const uint64_t ad = tc::smem_desc(a0 + kk * 256, lbo, sbo);
                    const uint64_t bd = tc::smem_desc(b0 + kk * 256, lbo, sbo);
                    tc::mma_bf16(tmem, ad, bd, idesc, k0 > 0 || kk > 0);
                }
                tc::mma_commit(&bar);
            }
            ok = tc::mbar_wait(&bar, phase, p.wait_limit);
            phase ^= 1u;
            if (!__syncthreads_and(ok))
            {
                ok = false;
                break;
            }
        }

        if (ok)
        {
            tc::fence_after_sync();
            const int row = m0 + tid;  // warp w holds TMEM lanes 32w..32w+31 = rows of this tile
            const uint32_t lane_base = tmem + (static_cast<uint32_t>(warp * 32) << 16);
            for (int c0 = 0; c0 < p.N; c0 += 32)
            {
                float v[32];
                tc::tmem_load32(lane_base + static_cast<uint32_t>(c0), v);
                const int cn = min(32, p.N - c0);
                if constexpr (EPI == kEpiStoreF32)
                {
                    float *dst = p.d_f32 + static_cast<size_t>(row) * p.N + c0;
                    for (int j = 0; j < cn; ++j)
                        dst[j] = v[j];
                }
                else
                {
                    __nv_bfloat16 *dst = p.d_bf16 + static_cast<size_t>(row) * p.N + c0;
                    for (int j = 0; j < cn; ++j)
                        dst[j] = __float2bfloat16_rn(fmaxf(__fadd_rn(v[j], p.bias[c0 + j]), 0.0f));
                }
            }
        }
        else if (tid == 0)
        {
            atomicExch(p.err, 1);
            // let any MMA still in flight finish before the accumulator is released
            tc::mbar_wait(&bar, phase ^ 1u, kWaitLimit);
        }
        tc::fence_before_sync();
        __syncthreads();
        if (warp == 0)
        {
            tc::fence_after_sync();
            tc::tmem_free(tmem, tcols);
        }
    }

    size_t gemm_smem_bytes(int N)
    {
        return static_cast<size_t>(128 + N) * kGemmKC * 2;
    }

    cudaError_t gemm_bf16(const GemmParams &p, int epi, cudaStream_t s)
    {
        const size_t smem = gemm_smem_bytes(p.N);
        const void *fn = epi == kEpiStoreF32 ? reinterpret_cast<const void *>(&gemm_bf16_kernel<kEpiStoreF32>)
                                             : reinterpret_cast<const void *>(&gemm_bf16_kernel<kEpiBiasReluBf16>);
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess)
            return e;
        if (epi == kEpiStoreF32)
            gemm_bf16_kernel<kEpiStoreF32><<<p.M / 128, 128, smem, s>>>(p);
        else
            gemm_bf16_kernel<kEpiBiasReluBf16><<<p.M / 128, 128, smem, s>>>(p);
        return cudaGetLastError();
    }
}  // namespace vg

using namespace vg;

extern "C" int vg_gemm_bf16_device(const void *a, const void *b, float *d, int M, int N, int K, int *err, void *stream)
{
    if (!a || !b || !d || !err || M <= 0 || M % 128 || N < 16 || N > 256 || N % 16 || K <= 0 || K % 16)
        return set_error(VG_ERR_ARG, "vg_gemm_bf16_device: need M % 128 == 0, N in 16..256 (multiple of 16), K % 16 == 0");
    GemmParams p{static_cast<const __nv_bfloat16 *>(a), static_cast<const __nv_bfloat16 *>(b), d, nullptr, nullptr, M, N, K, err};
    const cudaError_t e = gemm_bf16(p, kEpiStoreF32, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return set_error(VG_ERR_CUDA, std::string("gemm launch: ") + cudaGetErrorString(e));
    return VG_OK;
}

// =============================================================================================
// The MLP: features (sin, cos of each joint, zero-padded to a multiple of 16) -> 256 -> 256 -> 1
// with ReLU, BF16 weights and activations, FP32 accumulation and FP32 master weights (Adam).
// The forward and backward GEMMs run on gemm_bf16_kernel; small reductions on CUDA cores.

namespace vg
{
    constexpr int kHidden = 256;

    __global__ void features_kernel(const float *q, int n, int dim, int kin, __nv_bfloat16 *x, int rows)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= rows * kin)
            return;
        const int r = i / kin, c = i % kin;
        float v = 0.0f;
        if (r < n && c < 2 * dim)
        {
            const float a = q[static_cast<size_t>(r) * dim + (c >> 1)];
            v = (c & 1) ? cosf(a) : sinf(a);
        }
        x[i] = __float2bfloat16_rn(v);
    }

    // out[c][r] = in[r][c] for a [R][C] bf16 matrix
    __global__ void transpose_kernel(const __nv_bfloat16 *in, __nv_bfloat16 *out, int R, int C)
    {
        __shared__ __nv_bfloat16 tile[32][33];
        const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
        for (int k = threadIdx.y; k < 32; k += blockDim.y)
        {
            const int r = r0 + k, c = c0 + threadIdx.x;
            if (r < R && c < C)
                tile[k][threadIdx.x] = in[static_cast<size_t>(r) * C + c];
        }
        __syncthreads();
        for (int k = threadIdx.y; k < 32; k += blockDim.y)
        {
            const int c = c0 + k, r = r0 + threadIdx.x;
            if (r < R && c < C)
                out[static_cast<size_t>(c) * R + r] = tile[threadIdx.x][k];
        }
    }

    // z = H2 w3 + b3, p = sigmoid(z): one warp per row
    __global__ void head_kernel(const __nv_bfloat16 *h2, const float *w3, const float *b3, int rows, float *z, float *p)
    {
        const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
        const int lane = threadIdx.x & 31;
        if (row >= rows)
            return;
        float acc = 0.0f;
        for (int j = lane; j < kHidden; j += 32)
            acc = fmaf(__bfloat162float(h2[static_cast<size_t>(row) * kHidden + j]), w3[j], acc);
        for (int o = 16; o > 0; o >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0)
        {
            const float zz = acc + b3[0];
            if (z)
                z[row] = zz;
            p[row] = 1.0f / (1.0f + expf(-zz));
        }
    }

    // Binary cross-entropy on the logit: dz = (p - y) / n (rows >= n contribute nothing);
    // dH2 = dz w3 masked by H2 > 0 (bf16); loss accumulated into *loss.
    __global__ void head_backward_kernel(const __nv_bfloat16 *h2, const float *w3, const float *p, const float *z,
                                         const uint8_t *valid, int n, int rows, float *dz, __nv_bfloat16 *dh2, float *loss)
    {
        const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
        const int lane = threadIdx.x & 31;
        if (row >= rows)
            return;
        float g = 0.0f;
        if (row < n)
        {
            const float y = valid[row] ? 0.0f : 1.0f;  // label: 1 = in collision
            g = (p[row] - y) / static_cast<float>(n);
            if (lane == 0)
            {
                const float zz = z[row];
                // log(1 + exp(z)) - y z, evaluated stably
                const float l = fmaxf(zz, 0.0f) - zz * y + log1pf(expf(-fabsf(zz)));
                atomicAdd(loss, l / static_cast<float>(n));
            }
        }
        if (lane == 0)
            dz[row] = g;
        for (int j = lane; j < kHidden; j += 32)
        {
            const float h = __bfloat162float(h2[static_cast<size_t>(row) * kHidden + j]);
            dh2[static_cast<size_t>(row) * kHidden + j] = __float2bfloat16_rn(h > 0.0f ? g * w3[j] : 0.0f);
        }
    }

    // out[j] = sum_r a[r][j] * (w ? w[r] : 1) over rows, for a [rows][cols] matrix (bf16 or f32).
    // Block (32, 32): threadIdx.x picks the column of a 32-column group (coalesced loads),
    // threadIdx.y the row phase; a fixed-order reduction keeps the sums deterministic.
    template <typename T>
    __global__ void colsum_kernel(const T *a, const float *w, int rows, int cols, float *out)
    {
        const int j = blockIdx.x * 32 + threadIdx.x;
        float acc = 0.0f;
        if (j < cols)
        {
            for (int r = threadIdx.y; r < rows; r += 32)
            {
                float v;
                if constexpr (sizeof(T) == 2)
                    v = __bfloat162float(a[static_cast<size_t>(r) * cols + j]);
                else
                    v = a[static_cast<size_t>(r) * cols + j];
                acc = fmaf(v, w ? w[r] : 1.0f, acc);
            }
        }
        __shared__ float red[32][33];
        red[threadIdx.y][threadIdx.x] = acc;
        __syncthreads();
        if (threadIdx.y == 0 && j < cols)
        {
            float sum = 0.0f;
            for (int k = 0; k < 32; ++k)
                sum += red[k][threadIdx.x];
            out[j] = sum;
        }
    }

    // dH1 = (dH2 W2) masked by H1 > 0, as bf16
    __global__ void relu_mask_kernel(const float *g, const __nv_bfloat16 *h, int count, __nv_bfloat16 *out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i < count)
            out[i] = __float2bfloat16_rn(__bfloat162float(h[i]) > 0.0f ? g[i] : 0.0f);
    }

    // Adam on FP32 master weights, writing the BF16 copy the GEMMs read (when given)
    __global__ void adam_kernel(float *w, const float *g, float *m, float *v, int count, float lr, float b1, float b2,
                                float eps, float c1, float c2, __nv_bfloat16 *wb)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= count)
            return;
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb)
            wb[i] = __float2bfloat16_rn(wi);
    }

    __global__ void to_bf16_kernel(const float *in, __nv_bfloat16 *out, int count)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i < count)
            out[i] = __float2bfloat16_rn(in[i]);
    }
}  // namespace vg

// Parameter blocks, in the order vg_mlp_get_params/set_params use.
struct vg_mlp
{
    int kin = 16;  // padded input width
    int dim = 7;
    // fp32 masters: W1 [256][kin], b1 [256], W2 [256][256], b2 [256], w3 [256], b3 [1]
    float *w = nullptr;
    float *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *w1b = nullptr, *w2b = nullptr, *w2tb = nullptr;
    int step = 0;
    // workspace for `cap` rows
    int cap = 0;
    __nv_bfloat16 *x = nullptr, *h1 = nullptr, *h2 = nullptr, *dh2 = nullptr, *dh1 = nullptr, *t0 = nullptr, *t1 = nullptr;
    float *f32 = nullptr, *z = nullptr, *p = nullptr, *dz = nullptr, *loss = nullptr;
    int *err = nullptr;
    uint32_t wait_limit = vg::kWaitLimit;  // vg_mlp_set_wait_limit
    float *scores = nullptr;  // probe scores of the last learned edge check
    size_t scores_cap = 0;

    size_t n_w1() const { return static_cast<size_t>(vg::kHidden) * kin; }
    size_t count() const { return n_w1() + 256 + 256 * 256 + 256 + 256 + 1; }
    float *W1() const { return w; }
    float *B1() const { return w + n_w1(); }
    float *W2() const { return B1() + 256; }
    float *B2() const { return W2() + 256 * 256; }
    float *W3() const { return B2() + 256; }
    float *B3() const { return W3() + 256; }
    float *G(float *base, float *part) const { return base + (part - w); }
};

namespace vg
{
    static int mlp_reserve(vg_mlp *m, int rows)
    {
        if (rows <= m->cap)
            return VG_OK;
        void *old[] = {m->x, m->h1, m->h2, m->dh2, m->dh1, m->t0, m->t1, m->f32, m->z, m->p, m->dz};
        for (void *o : old)
            if (o)
                cudaFree(o);
        const size_t H = static_cast<size_t>(rows) * kHidden;
        cudaError_t e = cudaSuccess;
        auto get = [&](void **ptr, size_t bytes) {
            if (e == cudaSuccess)
                e = cudaMalloc(ptr, bytes);
        };
        get(reinterpret_cast<void **>(&m->x), static_cast<size_t>(rows) * m->kin * 2);
        get(reinterpret_cast<void **>(&m->h1), H * 2);
        get(reinterpret_cast<void **>(&m->h2), H * 2);
        get(reinterpret_cast<void **>(&m->dh2), H * 2);
        get(reinterpret_cast<void **>(&m->dh1), H * 2);
        get(reinterpret_cast<void **>(&m->t0), H * 2);
        get(reinterpret_cast<void **>(&m->t1), H * 2);
        get(reinterpret_cast<void **>(&m->f32), H * 4);
        get(reinterpret_cast<void **>(&m->z), static_cast<size_t>(rows) * 4);
        get(reinterpret_cast<void **>(&m->p), static_cast<size_t>(rows) * 4);
        get(reinterpret_cast<void **>(&m->dz), static_cast<size_t>(rows) * 4);
        if (e != cudaSuccess)
        {
            m->cap = 0;
            return set_error(VG_ERR_NOMEM, std::string("MLP workspace: ") + cudaGetErrorString(e));
        }
        m->cap = rows;
        return VG_OK;
    }

    static void sync_bf16(vg_mlp *m, cudaStream_t s)
    {
        to_bf16_kernel<<<(m->n_w1() + 255) / 256, 256, 0, s>>>(m->W1(), m->w1b, static_cast<int>(m->n_w1()));
        to_bf16_kernel<<<256, 256, 0, s>>>(m->W2(), m->w2b, 256 * 256);
    }

    // forward for `rows` rows (a multiple of 128) of configurations q[n][dim]; p receives
    // collision probabilities
    static int mlp_forward(vg_mlp *m, const float *q, int n, int rows, cudaStream_t s)
    {
        features_kernel<<<(rows * m->kin + 255) / 256, 256, 0, s>>>(q, n, m->dim, m->kin, m->x, rows);
        GemmParams g1{m->x, m->w1b, nullptr, m->h1, m->B1(), rows, kHidden, m->kin, m->err};
        g1.wait_limit = m->wait_limit;
        cudaError_t e = gemm_bf16(g1, kEpiBiasReluBf16, s);
        GemmParams g2{m->h1, m->w2b, nullptr, m->h2, m->B2(), rows, kHidden, kHidden, m->err};
        g2.wait_limit = m->wait_limit;
        if (e == cudaSuccess)
            e = gemm_bf16(g2, kEpiBiasReluBf16, s);
        if (e == cudaSuccess)
        {
            head_kernel<<<(rows + 7) / 8, 256, 0, s>>>(m->h2, m->W3(), m->B3(), rows, m->z, m->p);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess)
            return set_error(VG_ERR_CUDA, std::string("MLP forward: ") + cudaGetErrorString(e));
        return VG_OK;
    }

    // backward for a batch already run forward: gradients into m->grad; loss added to m->loss
    static int mlp_backward(vg_mlp *m, const uint8_t *valid, int n, int rows, cudaStream_t s)
    {
        float *gr = m->grad;
        head_backward_kernel<<<(rows + 7) / 8, 256, 0, s>>>(m->h2, m->W3(), m->p, m->z, valid, n, rows, m->dz, m->dh2, m->loss);
        colsum_kernel<__nv_bfloat16><<<kHidden / 32, dim3(32, 32), 0, s>>>(m->h2, m->dz, rows, kHidden, m->G(gr, m->W3()));  // dw3
        colsum_kernel<float><<<1, dim3(32, 32), 0, s>>>(m->dz, nullptr, rows, 1, m->G(gr, m->B3()));                     // db3
        colsum_kernel<__nv_bfloat16><<<kHidden / 32, dim3(32, 32), 0, s>>>(m->dh2, nullptr, rows, kHidden, m->G(gr, m->B2()));  // db2
        // dW2[j][i] = sum_r dH2[r][j] H1[r][i]
        const dim3 tb(32, 8);
        transpose_kernel<<<dim3(kHidden / 32, rows / 32), tb, 0, s>>>(m->dh2, m->t0, rows, kHidden);
        transpose_kernel<<<dim3(kHidden / 32, rows / 32), tb, 0, s>>>(m->h1, m->t1, rows, kHidden);
        GemmParams gw2{m->t0, m->t1, m->G(gr, m->W2()), nullptr, nullptr, kHidden, kHidden, rows, m->err};
        gw2.wait_limit = m->wait_limit;
        cudaError_t e = gemm_bf16(gw2, kEpiStoreF32, s);
        // dH1 = (dH2 W2) * (H1 > 0): B operand is W2^T as [i][j]
        GemmParams gh1{m->dh2, m->w2tb, m->f32, nullptr, nullptr, rows, kHidden, kHidden, m->err};
        gh1.wait_limit = m->wait_limit;
        if (e == cudaSuccess)
            e = gemm_bf16(gh1, kEpiStoreF32, s);
        if (e != cudaSuccess)
            return set_error(VG_ERR_CUDA, std::string("MLP backward: ") + cudaGetErrorString(e));
        relu_mask_kernel<<<(rows * kHidden + 255) / 256, 256, 0, s>>>(m->f32, m->h1, rows * kHidden, m->dh1);
        colsum_kernel<__nv_bfloat16><<<kHidden / 32, dim3(32, 32), 0, s>>>(m->dh1, nullptr, rows, kHidden, m->G(gr, m->B1()));  // db1
        // dW1[i][c] = sum_r dH1[r][i] X[r][c]
        transpose_kernel<<<dim3(kHidden / 32, rows / 32), tb, 0, s>>>(m->dh1, m->t0, rows, kHidden);
        transpose_kernel<<<dim3((m->kin + 31) / 32, rows / 32), tb, 0, s>>>(m->x, m->t1, rows, m->kin);
        GemmParams gw1{m->t0, m->t1, m->G(gr, m->W1()), nullptr, nullptr, kHidden, m->kin, rows, m->err};
        gw1.wait_limit = m->wait_limit;
        e = gemm_bf16(gw1, kEpiStoreF32, s);
        if (e != cudaSuccess)
            return set_error(VG_ERR_CUDA, std::string("MLP backward: ") + cudaGetErrorString(e));
        return VG_OK;
    }

    static void refresh_w2t(vg_mlp *m, cudaStream_t s)
    {
        // W2^T as bf16 [i][j] for the dH1 GEMM
        transpose_kernel<<<dim3(kHidden / 32, kHidden / 32), dim3(32, 8), 0, s>>>(m->w2b, m->w2tb, kHidden, kHidden);
    }

    static int mlp_check_err(vg_mlp *m)
    {
        int err = 0;
        cudaMemcpy(&err, m->err, sizeof(int), cudaMemcpyDeviceToHost);
        if (err)
            return set_error(VG_ERR_CUDA, "MLP: a tensor-core kernel gave up waiting for its MMAs");
        return VG_OK;
    }
}  // namespace vg

extern "C" {

size_t vg_mlp_param_count(int dim)
{
    vg_mlp m;
    m.kin = ((2 * dim + 15) / 16) * 16;
    return m.count();
}

vg_mlp *vg_mlp_create(int dim, uint64_t seed)
{
    if (dim < 1 || dim > 32)
    {
        set_error(VG_ERR_ARG, "vg_mlp_create: dim must be 1..32");
        return nullptr;
    }
    vg_mlp *m = new vg_mlp();
    m->dim = dim;
    m->kin = ((2 * dim + 15) / 16) * 16;
    const size_t n = m->count();
    cudaError_t e = cudaMalloc(&m->w, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&m->grad, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&m->m1, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&m->m2, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&m->w1b, m->n_w1() * 2);
    if (e == cudaSuccess) e = cudaMalloc(&m->w2b, 256 * 256 * 2);
    if (e == cudaSuccess) e = cudaMalloc(&m->w2tb, 256 * 256 * 2);
    if (e == cudaSuccess) e = cudaMalloc(&m->loss, 4);
    if (e == cudaSuccess) e = cudaMalloc(&m->err, 4);
    if (e != cudaSuccess)
    {
        set_error(VG_ERR_NOMEM, std::string("vg_mlp_create: ") + cudaGetErrorString(e));
        vg_mlp_destroy(m);
        return nullptr;
    }
    // He initialisation from a splitmix64 stream; biases 0
    std::vector<float> h(n, 0.0f);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto uniform = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t zz = st;
        zz = (zz ^ (zz >> 30)) * 0xBF58476D1CE4E5B9ull;
        zz = (zz ^ (zz >> 27)) * 0x94D049BB133111EBull;
        zz ^= zz >> 31;
        return static_cast<float>((zz >> 11) * (1.0 / 9007199254740992.0));
    };
    auto fill = [&](float *dst, size_t cnt, float fan_in) {
        const float a = std::sqrt(6.0f / fan_in);
        for (size_t i = 0; i < cnt; ++i)
            dst[i] = (2.0f * uniform() - 1.0f) * a;
    };
    fill(h.data(), m->n_w1(), static_cast<float>(2 * dim));
    for (size_t r = 0; r < 256; ++r)  // padded feature columns carry no weight
        for (int c = 2 * dim; c < m->kin; ++c)
            h[r * m->kin + c] = 0.0f;
    fill(h.data() + (m->W2() - m->w), 256 * 256, 256.0f);
    fill(h.data() + (m->W3() - m->w), 256, 256.0f);
    cudaMemcpy(m->w, h.data(), n * 4, cudaMemcpyHostToDevice);
    cudaMemset(m->m1, 0, n * 4);
    cudaMemset(m->m2, 0, n * 4);
    cudaMemset(m->err, 0, 4);
    sync_bf16(m, 0);
    refresh_w2t(m, 0);
    cudaDeviceSynchronize();
    return m;
}

void vg_mlp_destroy(vg_mlp *m)
{
    if (!m)
        return;
    void *ptrs[] = {m->w, m->grad, m->m1, m->m2, m->w1b, m->w2b, m->w2tb, m->x, m->h1, m->h2, m->dh2, m->dh1, m->t0, m->t1,
                    m->f32, m->z, m->p, m->dz, m->loss, m->err, m->scores};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    delete m;
}

int vg_mlp_get_params(const vg_mlp *m, float *out)
{
    if (!m || !out)
        return set_error(VG_ERR_ARG, "vg_mlp_get_params: bad argument");
    if (cudaMemcpy(out, m->w, m->count() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(VG_ERR_CUDA, "vg_mlp_get_params: copy failed");
    return VG_OK;
}

int vg_mlp_set_params(vg_mlp *m, const float *in)
{
    if (!m || !in)
        return set_error(VG_ERR_ARG, "vg_mlp_set_params: bad argument");
    if (cudaMemcpy(m->w, in, m->count() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return set_error(VG_ERR_CUDA, "vg_mlp_set_params: copy failed");
    sync_bf16(m, 0);
    refresh_w2t(m, 0);
    return cudaDeviceSynchronize() == cudaSuccess ? VG_OK : set_error(VG_ERR_CUDA, "vg_mlp_set_params");
}

int vg_mlp_predict_device(vg_mlp *m, const float *q, size_t n, float *p_out, void *stream)
{
    if (!m || (n && (!q || !p_out)))
        return set_error(VG_ERR_ARG, "vg_mlp_predict_device: bad argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t done = 0;
    const size_t chunk = 1 << 16;
    while (done < n)
    {
        const int cnt = static_cast<int>(std::min(chunk, n - done));
        const int rows = (cnt + 127) / 128 * 128;
        if (int rc = mlp_reserve(m, rows))
            return rc;
        if (int rc = mlp_forward(m, q + done * m->dim, cnt, rows, s))
            return rc;
        if (cudaMemcpyAsync(p_out + done, m->p, cnt * 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return set_error(VG_ERR_CUDA, "vg_mlp_predict_device: copy");
        done += cnt;
    }
    return VG_OK;
}

// One forward + backward on n <= 65536 configurations; gradients (count floats, parameter
// order), the loss and the bf16 features (rows x kin, as floats) are returned to the host.
int vg_mlp_gradients(vg_mlp *m, const float *q_dev, const uint8_t *valid_dev, size_t n, float *grads, float *loss,
                     float *features)
{
    if (!m || !q_dev || !valid_dev || n == 0 || n > 65536 || !grads || !loss)
        return set_error(VG_ERR_ARG, "vg_mlp_gradients: bad argument");
    const int rows = static_cast<int>((n + 127) / 128 * 128);
    if (int rc = mlp_reserve(m, rows))
        return rc;
    cudaMemset(m->loss, 0, 4);
    if (int rc = mlp_forward(m, q_dev, static_cast<int>(n), rows, 0))
        return rc;
    if (int rc = mlp_backward(m, valid_dev, static_cast<int>(n), rows, 0))
        return rc;
    if (cudaDeviceSynchronize() != cudaSuccess)
        return set_error(VG_ERR_CUDA, "vg_mlp_gradients: kernel failure");
    if (int rc = mlp_check_err(m))
        return rc;
    cudaMemcpy(grads, m->grad, m->count() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(loss, m->loss, 4, cudaMemcpyDeviceToHost);
    if (features)
    {
        std::vector<__nv_bfloat16> xb(static_cast<size_t>(rows) * m->kin);
        cudaMemcpy(xb.data(), m->x, xb.size() * 2, cudaMemcpyDeviceToHost);
        for (size_t i = 0; i < n * m->kin; ++i)
            features[i] = __bfloat162float(xb[i]);
    }
    return VG_OK;
}

// Adam training on n labelled configurations (q_dev [n][dim], valid_dev[n]: 1 = collision free),
// `epochs` passes in minibatches of `batch` rows (a multiple of 128).  losses (host, may be NULL)
// receives the mean loss of each epoch.
int vg_mlp_train_device(vg_mlp *m, const float *q_dev, const uint8_t *valid_dev, size_t n, int epochs, int batch,
                        float lr, float *losses, void *stream)
{
    if (!m || !q_dev || !valid_dev || n < 128 || epochs < 1 || batch < 128 || batch % 128 || !(lr > 0))
        return set_error(VG_ERR_ARG, "vg_mlp_train_device: bad argument (batch must be a multiple of 128)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (int rc = mlp_reserve(m, batch))
        return rc;
    const size_t steps = n / batch;
    for (int ep = 0; ep < epochs; ++ep)
    {
        cudaMemsetAsync(m->loss, 0, 4, s);
        for (size_t st = 0; st < steps; ++st)
        {
            const size_t off = st * batch;
            if (int rc = mlp_forward(m, q_dev + off * m->dim, batch, batch, s))
                return rc;
            if (int rc = mlp_backward(m, valid_dev + off, batch, batch, s))
                return rc;
            ++m->step;
            if (ep == 0 && st == 0)
            {
                // the first step shows whether the tensor-core kernels work on this device
                if (cudaStreamSynchronize(s) != cudaSuccess)
                    return set_error(VG_ERR_CUDA, "vg_mlp_train_device: kernel failure");
                if (int rc = mlp_check_err(m))
                    return rc;
            }
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.0f - std::pow(b1, static_cast<float>(m->step));
            const float c2 = 1.0f - std::pow(b2, static_cast<float>(m->step));
            const int cnt = static_cast<int>(m->count());
            adam_kernel<<<(cnt + 255) / 256, 256, 0, s>>>(m->w, m->grad, m->m1, m->m2, cnt, lr, b1, b2, 1e-8f, c1, c2, nullptr);
            sync_bf16(m, s);
            refresh_w2t(m, s);
        }
        if (losses)
        {
            float l = 0;
            cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            losses[ep] = l / static_cast<float>(steps);
        }
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
        return set_error(VG_ERR_CUDA, "vg_mlp_train_device: kernel failure");
    return mlp_check_err(m);
}

}  // extern "C"

// =============================================================================================
// Fused inference: one persistent CTA per SM keeps W1 and W2 (BF16, core-matrix layout) in
// shared memory and, per 128-row tile, computes features -> L1 (one tcgen05 MMA group into half
// of the TMEM columns) -> bias+ReLU -> BF16 H1 in shared memory -> L2 (the same half) ->
// bias+ReLU -> BF16 H2 -> dot with w3 in registers.  Nothing but the scores leaves the SM.
//
// Row g scores a state: with b == nullptr, configuration a[g]; otherwise probe p = g % P of edge
// e = g / P, the state a + (p + 0.5) / P (b - a).

namespace vg
{
    // bf16x2 {lo: relu(v.x), hi: relu(v.y)}, each rounded to nearest
    __device__ __forceinline__ uint32_t relu_bf16x2(float2 v)
    {
        uint32_t h;
        asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(v.y), "f"(v.x));
        return h;
    }

    // the two BF16 halves of h as floats {lo, hi}
    __device__ __forceinline__ float2 bf16x2_to_float2(uint32_t h)
    {
        return make_float2(__uint_as_float(h << 16), __uint_as_float(h & 0xffff0000u));
    }

    struct InferParams
    {
        const float *a;
        const float *b;
        int probes;      // P (1 with b == nullptr)
        long long rows;  // n * P
        int dim;
        const __nv_bfloat16 *w1;  // [256][KIN]
        const __nv_bfloat16 *w2;  // [256][256]
        const float *b1, *b2, *w3, *b3;
        float *out;               // [rows]
        int probability;          // 1: sigmoid(z), 0: z
        int *err;
        uint32_t wait_limit = kWaitLimit;  // as GemmParams::wait_limit
    };

    template <int KIN>
    constexpr size_t infer_smem_bytes()
    {
        return static_cast<size_t>(kHidden) * KIN * 2      // W1
               + static_cast<size_t>(kHidden) * kHidden * 2  // W2
               + 128u * KIN * 2                              // X tile
               + 128u * kHidden * 2                          // H1 tile
               + 3u * kHidden * 4;                           // b1, b2, w3
    }

    // Threads of the fused inference kernel: 16 warps.  Warp w reads TMEM lanes 32 (w % 4) ..
    // 32 (w % 4) + 31 (the rows of its lane quarter, as tcgen05.ld allows) and columns
    // 64 (w / 4) .. 64 (w / 4) + 63 of each 256-column accumulator, so four warps share each
    // quarter's epilogue work and every scheduler has four warps to switch between.
    constexpr int kInferThreads = 512;

    // Per 128-row tile: layer 1 (X W1^T into one half of the 512 TMEM columns), bias + ReLU to
    // BF16 in shared memory (H1), layer 2 (H1 W2^T into the same half), bias + ReLU + dot with
    // w3.  Tiles alternate halves and are pipelined: the next tile's features are computed while
    // this tile's layer 2 runs, and the next tile's layer 2 runs while this tile's layer-2
    // epilogue reads the other half.  One mbarrier per layer; every wait is bounded, and a kernel
    // that gives up waits (with the default limit) for the MMAs it issued before it frees the
    // tensor memory.
    template <int KIN>
    __global__ void __launch_bounds__(kInferThreads, 1) mlp_infer_kernel(const InferParams p)
    {
        extern __shared__ __align__(1024) unsigned char infer_smem[];
        __shared__ uint64_t bar1, bar2;
        __shared__ uint32_t tmem_slot;
        __shared__ float zpart[4][128];  // partial dot products per column slice and row
        unsigned char *sw1 = infer_smem;
        unsigned char *sw2 = sw1 + kHidden * KIN * 2;
        unsigned char *sx = sw2 + kHidden * kHidden * 2;
        unsigned char *sh = sx + 128 * KIN * 2;
        float *sb1 = reinterpret_cast<float *>(sh + 128 * kHidden * 2);
        float *sb2 = sb1 + kHidden;
        float *sw3 = sb2 + kHidden;
        const int tid = threadIdx.x;
        const int warp = tid >> 5;
        const int quarter = warp & 3;               // TMEM lane quarter
        const int slice = warp >> 2;                // 64-column slice
        const int row = 32 * quarter + (tid & 31);  // tile row of this thread in the epilogues
        __shared__ int skip;

        if (tid == 0)
            skip = *static_cast<volatile int *>(p.err);
        __syncthreads();
        if (skip)
            return;
        if (warp == 0)
            tc::tmem_alloc(&tmem_slot, 512);
        if (tid == 0)
        {
            tc::mbar_init(&bar1, 1);
            tc::mbar_init(&bar2, 1);
        }
        // weights into core-matrix layout, 16-byte units
        for (int u = tid; u < kHidden * (KIN / 8); u += kInferThreads)
        {
            const int r = u / (KIN / 8), g = u % (KIN / 8);
            *reinterpret_cast<uint4 *>(sw1 + tc::tile_offset(r, 8 * g, KIN)) =
                *reinterpret_cast<const uint4 *>(p.w1 + static_cast<size_t>(r) * KIN + 8 * g);
        }
        for (int u = tid; u < kHidden * (kHidden / 8); u += kInferThreads)
        {
            const int r = u / (kHidden / 8), g = u % (kHidden / 8);
            *reinterpret_cast<uint4 *>(sw2 + tc::tile_offset(r, 8 * g, kHidden)) =
                *reinterpret_cast<const uint4 *>(p.w2 + static_cast<size_t>(r) * kHidden + 8 * g);
        }
        for (int j = tid; j < kHidden; j += kInferThreads)
        {
            sb1[j] = p.b1[j];
            sb2[j] = p.b2[j];
            sw3[j] = p.w3[j];
        }
        const float b3 = p.b3[0];
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tmem = tmem_slot;
        const uint32_t lane_base = tmem + (static_cast<uint32_t>(quarter * 32) << 16);
        const int c_lo = 64 * slice;  // this warp's first accumulator column
        const uint32_t idesc = tc::idesc_bf16_f32(128, kHidden);
        uint32_t ph1 = 0, ph2 = 0;     // phases the next waits on bar1 / bar2 expect
        bool pend1 = false, pend2 = false;  // an MMA group committed to bar1 / bar2 and not yet waited for
        const long long tiles = (p.rows + 127) / 128;

        // features of a tile: item i (row i % 128, joint d = i / 128) writes sin and cos of joint
        // d of its row's state (zeros past the robot's joints); every thread takes KIN / 8 items,
        // all of one row, so that all 16 warps share the sines and cosines.  A tile's first row
        // g0 = e0 P + r0 is carried from tile to tile (tiles advance by a fixed number of rows),
        // which leaves one 32-bit division per thread and tile, and each call loads the joint
        // values of the CTA's following tile, so that their latency passes under a whole tile.
        constexpr int kItems = KIN / 8;
        const int frow = tid & 127;
        const long long step_rows = static_cast<long long>(gridDim.x) * 128;
        const long long step_e = step_rows / p.probes;
        const int step_r = static_cast<int>(step_rows - step_e * p.probes);
        long long ftile = blockIdx.x;  // the tile the loaded values belong to
        long long e0 = ftile * 128 / p.probes;
        int r0 = static_cast<int>(ftile * 128 - e0 * p.probes);
        float in_a[kItems], in_v[kItems], in_t = 0.0f;
        bool in_row = false;
        auto load_inputs = [&]() {
            const int loc = r0 + frow;
            const long long e = e0 + loc / p.probes;
            in_t = (static_cast<float>(loc % p.probes) + 0.5f) / static_cast<float>(p.probes);
            in_row = ftile * 128 + frow < p.rows;
#pragma unroll
            for (int k = 0; k < kItems; ++k)
            {
                const int d = (tid >> 7) + 4 * k;
                in_a[k] = 0.0f;
                in_v[k] = 0.0f;
                if (in_row && d < p.dim)
                {
                    in_a[k] = p.a[e * p.dim + d];
                    if (p.b)
                        in_v[k] = p.b[e * p.dim + d] - in_a[k];
                }
            }
        };
        auto features = [&]() {
#pragma unroll
            for (int k = 0; k < kItems; ++k)
            {
                const int d = (tid >> 7) + 4 * k;
                __nv_bfloat162 f = __floats2bfloat162_rn(0.0f, 0.0f);
                if (in_row && d < p.dim)
                {
                    const float q = p.b ? fmaf(in_v[k], in_t, in_a[k]) : in_a[k];
                    f = __floats2bfloat162_rn(sinf(q), cosf(q));
                }
                *reinterpret_cast<__nv_bfloat162 *>(sx + tc::tile_offset(frow, 2 * d, KIN)) = f;
            }
            // the CTA's next tile
            ftile += gridDim.x;
            e0 += step_e;
            r0 += step_r;
            if (r0 >= p.probes)
            {
                r0 -= p.probes;
                ++e0;
            }
            if (ftile < tiles)
                load_inputs();
        };
        auto issue_layer1 = [&](uint32_t acc) {
            if (tid == 0)
            {
                tc::fence_after_sync();
                const uint32_t x0 = tc::smem_u32(sx), w0 = tc::smem_u32(sw1);
#pragma unroll
                for (int kk = 0; kk < KIN / 16; ++kk)
                    tc::mma_bf16(tmem + acc, tc::smem_desc(x0 + kk * 256, 128, (KIN / 8) * 128),
                                 tc::smem_desc(w0 + kk * 256, 128, (KIN / 8) * 128), idesc, kk > 0);
                tc::mma_commit(&bar1);
            }
            pend1 = true;
        };
        auto issue_layer2 = [&](uint32_t acc) {
            if (tid == 0)
            {
                tc::fence_after_sync();
                const uint32_t h0 = tc::smem_u32(sh), w0 = tc::smem_u32(sw2);
#pragma unroll 4
                for (int kk = 0; kk < kHidden / 16; ++kk)
                    tc::mma_bf16(tmem + acc, tc::smem_desc(h0 + kk * 256, 128, (kHidden / 8) * 128),
                                 tc::smem_desc(w0 + kk * 256, 128, (kHidden / 8) * 128), idesc, kk > 0);
                tc::mma_commit(&bar2);
            }
            pend2 = true;
        };
        // bounded wait for the group committed to bar; every thread takes the same decision
        auto wait_for = [&](uint64_t *bar, uint32_t &ph, bool &pend) {
            bool ok = tc::mbar_wait(bar, ph, p.wait_limit);
            ok = __syncthreads_and(ok) != 0;
            if (ok)
            {
                ph ^= 1u;
                pend = false;
                tc::fence_after_sync();
            }
            return ok;
        };
        // H1 = bf16(relu(D1 + b1)) into shared memory: this warp's rows and column slice.  Two
        // columns per instruction: packed FP32 adds, and one conversion that rounds both sums to
        // BF16 and clamps them at zero (ReLU commutes with round-to-nearest).
        auto epilogue1 = [&](uint32_t acc) {
#pragma unroll
            for (int c0 = c_lo; c0 < c_lo + 64; c0 += 32)
            {
                float v[32];
                tc::tmem_load32(lane_base + acc + static_cast<uint32_t>(c0), v);
#pragma unroll
                for (int j = 0; j < 32; j += 8)
                {
                    const float4 ba = *reinterpret_cast<const float4 *>(sb1 + c0 + j);
                    const float4 bb = *reinterpret_cast<const float4 *>(sb1 + c0 + j + 4);
                    __align__(16) uint32_t h[4];
                    h[0] = relu_bf16x2(__fadd2_rn(make_float2(v[j], v[j + 1]), make_float2(ba.x, ba.y)));
                    h[1] = relu_bf16x2(__fadd2_rn(make_float2(v[j + 2], v[j + 3]), make_float2(ba.z, ba.w)));
                    h[2] = relu_bf16x2(__fadd2_rn(make_float2(v[j + 4], v[j + 5]), make_float2(bb.x, bb.y)));
                    h[3] = relu_bf16x2(__fadd2_rn(make_float2(v[j + 6], v[j + 7]), make_float2(bb.z, bb.w)));
                    *reinterpret_cast<uint4 *>(sh + tc::tile_offset(row, c0 + j, kHidden)) = *reinterpret_cast<const uint4 *>(h);
                }
            }
            tc::fence_smem_to_async();
            tc::fence_before_sync();
            __syncthreads();
        };
        // z = bf16(relu(D2 + b2)) . w3 + b3: partial sums over this warp's 64 columns (even and
        // odd columns in the two halves of packed FP32 multiply-adds), added slice by slice
        auto epilogue2 = [&](long long tile, uint32_t acc) {
            float2 z2 = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int c0 = c_lo; c0 < c_lo + 64; c0 += 32)
            {
                float v[32];
                tc::tmem_load32(lane_base + acc + static_cast<uint32_t>(c0), v);
#pragma unroll
                for (int j = 0; j < 32; j += 4)
                {
                    const float4 bb = *reinterpret_cast<const float4 *>(sb2 + c0 + j);
                    const float4 ww = *reinterpret_cast<const float4 *>(sw3 + c0 + j);
                    const uint32_t h0 = relu_bf16x2(__fadd2_rn(make_float2(v[j], v[j + 1]), make_float2(bb.x, bb.y)));
                    const uint32_t h1 = relu_bf16x2(__fadd2_rn(make_float2(v[j + 2], v[j + 3]), make_float2(bb.z, bb.w)));
                    z2 = __ffma2_rn(bf16x2_to_float2(h0), make_float2(ww.x, ww.y), z2);
                    z2 = __ffma2_rn(bf16x2_to_float2(h1), make_float2(ww.z, ww.w), z2);
                }
            }
            const float z = __fadd_rn(z2.x, z2.y);
            zpart[slice][row] = z;
            tc::fence_before_sync();
            __syncthreads();
            if (slice == 0)
            {
                const long long g = tile * 128 + row;
                const float zz = ((zpart[0][row] + zpart[1][row]) + (zpart[2][row] + zpart[3][row])) + b3;
                if (g < p.rows)
                    p.out[g] = p.probability ? 1.0f / (1.0f + expf(-zz)) : zz;
            }
            // zpart is written again only after two more block-wide barriers
        };

        bool ok = true;
        long long tile = blockIdx.x;
        if (tile < tiles)
        {
            // Layer 1 and layer 2 of a tile share one half of the 512 accumulator columns, the
            // halves alternating from tile to tile: the next tile's layer 1, its epilogue and its
            // layer 2 go into the other half while this tile's layer-2 result waits, so the next
            // tile's layer 2 runs on the tensor core during this tile's layer-2 epilogue.
            uint32_t acc = 0;
            load_inputs();
            features();
            tc::fence_smem_to_async();
            tc::fence_before_sync();
            __syncthreads();
            issue_layer1(acc);
            ok = wait_for(&bar1, ph1, pend1);
            if (ok)
            {
                epilogue1(acc);
                issue_layer2(acc);
            }
            while (ok)
            {
                const long long next = tile + gridDim.x;
                const bool has_next = next < tiles;
                const uint32_t acc_next = acc ^ static_cast<uint32_t>(kHidden);
                if (has_next)
                {
                    features();  // the next tile's, while this tile's layer 2 runs
                }
                tc::fence_smem_to_async();
                tc::fence_before_sync();
                __syncthreads();
                ok = wait_for(&bar2, ph2, pend2);  // this tile's layer 2; H1 is free again
                if (!ok)
                    break;
                if (has_next)
                {
                    // the other half was last read by the previous tile's layer-2 epilogue
                    issue_layer1(acc_next);
                    ok = wait_for(&bar1, ph1, pend1);
                    if (!ok)
                        break;
                    epilogue1(acc_next);
                    issue_layer2(acc_next);  // runs during this tile's layer-2 epilogue
                }
                epilogue2(tile, acc);
                if (!has_next)
                    break;
                tile = next;
                acc = acc_next;
            }
        }
        if (!ok && tid == 0)
        {
            atomicExch(p.err, 1);
            // let the MMAs still in flight finish before the accumulator is released
            if (pend1)
                tc::mbar_wait(&bar1, ph1, kWaitLimit);
            if (pend2)
                tc::mbar_wait(&bar2, ph2, kWaitLimit);
        }
        tc::fence_before_sync();
        __syncthreads();
        if (warp == 0)
        {
            tc::fence_after_sync();
            tc::tmem_free(tmem, 512);
        }
    }

    static int mlp_infer(vg_mlp *m, const float *a, const float *b, int probes, long long rows, float *out, int probability,
                         cudaStream_t s)
    {
        if (rows == 0)
            return VG_OK;
        if (m->kin > 32)
            return set_error(VG_ERR_LIMIT, "MLP inference: at most 16 joints (32 sin/cos features)");
        InferParams ip{a, b, probes, rows, m->dim, m->w1b, m->w2b, m->B1(), m->B2(), m->W3(), m->B3(), out, probability, m->err};
        ip.wait_limit = m->wait_limit;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long tiles = (rows + 127) / 128;
        const int grid = static_cast<int>(std::min<long long>(tiles, sms));
        cudaError_t e;
        if (m->kin == 16)
        {
            const size_t smem = infer_smem_bytes<16>();
            e = cudaFuncSetAttribute(mlp_infer_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e == cudaSuccess)
            {
                mlp_infer_kernel<16><<<grid, kInferThreads, smem, s>>>(ip);
                e = cudaGetLastError();
            }
        }
        else
        {
            const size_t smem = infer_smem_bytes<32>();
            e = cudaFuncSetAttribute(mlp_infer_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e == cudaSuccess)
            {
                mlp_infer_kernel<32><<<grid, kInferThreads, smem, s>>>(ip);
                e = cudaGetLastError();
            }
        }
        if (e != cudaSuccess)
            return set_error(VG_ERR_CUDA, std::string("MLP inference: ") + cudaGetErrorString(e));
        return VG_OK;
    }
}  // namespace vg

extern "C" {

int vg_mlp_infer_device(vg_mlp *m, const float *q, size_t n, float *p_out, void *stream)
{
    if (!m || (n && (!q || !p_out)))
        return set_error(VG_ERR_ARG, "vg_mlp_infer_device: bad argument");
    return mlp_infer(m, q, nullptr, 1, static_cast<long long>(n), p_out, 1, static_cast<cudaStream_t>(stream));
}

int vg_mlp_score_edges_device(vg_mlp *m, const float *a, const float *b, size_t n, int probes, float *scores, void *stream)
{
    if (!m || (n && (!a || !b || !scores)) || probes < 1 || probes > 32)
        return set_error(VG_ERR_ARG, "vg_mlp_score_edges_device: bad argument (probes 1..32)");
    return mlp_infer(m, a, b, probes, static_cast<long long>(n) * probes, scores, 0, static_cast<cudaStream_t>(stream));
}

int vg_mlp_error(vg_mlp *m)
{
    if (!m)
        return set_error(VG_ERR_ARG, "vg_mlp_error: null");
    const int rc = mlp_check_err(m);
    if (rc != VG_OK)
    {
        // reported once: later calls on this handle run again
        cudaMemset(m->err, 0, sizeof(int));
        cudaDeviceSynchronize();
    }
    return rc;
}

int vg_mlp_set_wait_limit(vg_mlp *m, long long polls)
{
    if (!m || polls > 0x7fffffffLL)
        return set_error(VG_ERR_ARG, "vg_mlp_set_wait_limit: polls must be at most 2^31 - 1 (negative: the default)");
    m->wait_limit = polls < 0 ? kWaitLimit : static_cast<uint32_t>(polls);
    return VG_OK;
}

}  // extern "C"

extern "C" {

// Learned-order edge check: scores `probes` states per edge with the MLP (fused tcgen05
// inference) and checks each edge's blocks in the order those scores rank them.  Verdicts are
// those of vg_validate_motions_device.  The scores stay in the MLP's scratch (device memory,
// reallocated when a larger batch comes), so calls sharing one vg_mlp must not overlap.
int vg_validate_motions_learned_device(const char *robot, vg_env *env, vg_mlp *m, const float *a, const float *b, size_t n,
                                       int resolution, int probes, uint8_t *out, int32_t *blocks, void *stream)
{
    if (!m || probes < 1 || probes > 32)
        return set_error(VG_ERR_ARG, "vg_validate_motions_learned_device: bad argument (probes 1..32)");
    if (n == 0)
        return VG_OK;
    const size_t need = n * static_cast<size_t>(probes);
    if (need > m->scores_cap)
    {
        if (m->scores)
            cudaFree(m->scores);
        m->scores = nullptr;
        m->scores_cap = 0;
        if (cudaMalloc(&m->scores, need * sizeof(float)) != cudaSuccess)
            return set_error(VG_ERR_NOMEM, "vg_validate_motions_learned_device: scores buffer");
        m->scores_cap = need;
    }
    if (int rc = vg_mlp_score_edges_device(m, a, b, n, probes, m->scores, stream))
        return rc;
    return vg_validate_motions_scored_device(robot, env, a, b, n, resolution, m->scores, probes, out, blocks, stream);
}

}  // extern "C"
