// mlp.cu -- tensor-core (tcgen05, BF16 in / FP32 accumulate) kernels of the
// learned proposal for the energy-transfer draw.
//
// k_gemm_bf16 is the general product C = A B of the training step: A and B
// are read from FP32 arrays with arbitrary strides (so transposes cost
// nothing), rounded to BF16 while staged into shared memory in the K-major
// layout the tensor core reads, multiplied by tcgen05.mma into an FP32 TMEM
// accumulator, and read back with tcgen05.ld.  One CTA (one warpgroup) makes a
// 128 x 64 tile of C, K in chunks of 64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include "mc.cuh"
#include "tc.cuh"

namespace tk {

constexpr int GB_M = 128, GB_N = 64, GB_K = 64;
// 24 KB of operand tiles; asking for 48 KB keeps at most four CTAs (4 x 64
// TMEM columns of the 512) on an SM, so an allocation never waits long
constexpr int GB_SMEM = 48 * 1024;
constexpr long long kWaitCycles = 2000000000ll;   // about one second at 2 GHz

__global__ void __launch_bounds__(128) k_gemm_bf16(const float* __restrict__ A, long long as_m, long long as_k,
                                                   const float* __restrict__ B, long long bs_k, long long bs_n,
                                                   float* __restrict__ C, long long ldc, int M, int N, int K,
                                                   int accumulate, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sA = smem;                          // 128 x 64 BF16, K-major
    unsigned char* sB = smem + GB_M * GB_K * 2;        // 64 x 64 BF16 (rows = columns of C)
    uint64_t* mbar = (uint64_t*)(smem + (GB_M + GB_N) * GB_K * 2);
    uint32_t* tslot = (uint32_t*)(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * GB_M, n0 = blockIdx.y * GB_N;
    // split-K: CTA z takes the K chunks [kb, ke) and adds its part into C atomically
    const int kper = ((K + GB_K - 1) / GB_K + gridDim.z - 1) / gridDim.z * GB_K;
    const int kb = blockIdx.z * kper, ke = min(K, kb + kper);
    if (warp == 0) tc::tmem_alloc(tslot, GB_N);
    if (tid == 0) tc::mbar_init(mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = tc::idesc_bf16(GB_M, GB_N);
    uint32_t phase = 0;
    bool ok = true;
    int issued = 0;
    for (int k0 = kb; k0 < ke && ok; k0 += GB_K) {
        for (int e = tid; e < GB_M * GB_K; e += 128) {
            const int r = e / GB_K, k = e % GB_K, m = m0 + r, kk = k0 + k;
            const float v = (m < M && kk < ke) ? A[m * as_m + kk * as_k] : 0.f;
            *(__nv_bfloat16*)(sA + tc::kmaj_off(r, k, GB_K)) = __float2bfloat16_rn(v);
        }
        for (int e = tid; e < GB_N * GB_K; e += 128) {
            const int r = e / GB_K, k = e % GB_K, n = n0 + r, kk = k0 + k;
            const float v = (n < N && kk < ke) ? B[kk * bs_k + n * bs_n] : 0.f;
            *(__nv_bfloat16*)(sB + tc::kmaj_off(r, k, GB_K)) = __float2bfloat16_rn(v);
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
#pragma unroll
            for (int s = 0; s < GB_K / 16; ++s)
                tc::mma_bf16(tmem, tc::smem_desc(a0 + s * 256, 128, GB_K * 16), tc::smem_desc(b0 + s * 256, 128, GB_K * 16),
                             idesc, (k0 > kb || s > 0) ? 1u : 0u);
            tc::mma_commit(mbar);
        }
        ++issued;
        // the tiles are rewritten next round: wait for the MMAs that read them;
        // the CTA agrees on the outcome so every thread leaves the loop together
        const int late = __syncthreads_or(tc::mbar_wait(mbar, phase, kWaitCycles) ? 0 : 1);
        if (late) {
            ok = false;
            tc::mbar_wait(mbar, phase, kWaitCycles);   // give the MMAs in flight a second bounded wait
        }
        phase ^= 1u;
        tc::fence_after_sync();
    }
    if (ok) {
        const int r = warp * 32 + (tid & 31), m = m0 + r;
#pragma unroll
        for (int c = 0; c < GB_N; c += 16) {
            float v[16];
            if (issued) tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            else for (int j = 0; j < 16; ++j) v[j] = 0.f;
            if (m < M)
                for (int j = 0; j < 16; ++j) {
                    const int n = n0 + c + j;
                    if (n < N) {
                        float* p = C + m * ldc + n;
                        if (gridDim.z > 1) atomicAdd(p, v[j]);
                        else *p = accumulate ? *p + v[j] : v[j];
                    }
                }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, GB_N);
}

// splitk > 1: C must hold the value to add to (zero for a plain product)
int gemm_bf16(const float* A, long long as_m, long long as_k, const float* B, long long bs_k, long long bs_n, float* C,
              long long ldc, int M, int N, int K, int accumulate, int* derr, cudaStream_t s, int splitk = 1) {
    if (M <= 0 || N <= 0) return 0;
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_SMEM) != cudaSuccess)
            return -1;
        attr_set = true;
    }
    splitk = std::max(1, std::min(splitk, (K + GB_K - 1) / GB_K));
    dim3 grid((M + GB_M - 1) / GB_M, (N + GB_N - 1) / GB_N, splitk);
    k_gemm_bf16<<<grid, 128, GB_SMEM, s>>>(A, as_m, as_k, B, bs_k, bs_n, C, ldc, M, N, K, accumulate, derr);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---- the proposal network -------------------------------------------------------------
// Input (2): the energy mapped onto [-1, 1] over the network's log E range
// and the uniform of the draw through prop_u_feature.  Output (1): the bracket's position
// as a fraction of the cumulative row, (ih - 1 + w) / (len - 1), w the log-log
// position inside the bracket.  Hidden: 64, 64, SiLU.  Parameters (FP32
// master copy): W1[2][64], b1, W2[64][64] (in, out), b2, w3[64], b3.
constexpr int NP = 128 + 64 + 4096 + 64 + 64 + 1;
constexpr int OFF_W1 = 0, OFF_B1 = 128, OFF_W2 = 192, OFF_B2 = 4288, OFF_W3 = 4352, OFF_B3 = 4416;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float sg = 1.f / (1.f + __expf(-z));
    return sg * (1.f + z * (1.f - sg));
}

struct NetSpec {
    int hole;      // 0: electron shell k, 1: valence holes
    int k;         // compact shell whose per-shell MFP sets L_tot
    float lo, hi;  // log E range
};

// Training samples of one network from the FP32 tables: the exact bracket of
// sample_transfer / interp_transfer for (E, u), E log-uniform in [lo, hi].
__global__ void k_mlp_data(DevTabs<float> tb, NetSpec ns, uint64_t seed, uint32_t stream, long long n, float* X,
                           float* Tg) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t w[4];
    philox4x32((uint32_t)i, (uint32_t)(i >> 32), stream, 0x4D4C5050u, (uint32_t)seed, (uint32_t)(seed >> 32), w);
    const float a = ((float)(w[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float u = ((float)(w[1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float E = expf(ns.lo + a * (ns.hi - ns.lo));
    const float* Eg; int nE; const int* roff; const float* rL; float Ltot;
    if (ns.hole) {
        Eg = tb.hE; nE = tb.nH; roff = tb.hrow_off; rL = tb.hrow_L;
        Ltot = nfp1(Tab<float>{tb.hE, tb.hL + (size_t)ns.k * tb.nH, tb.nH}, E);
    } else {
        Eg = tb.elE; nE = tb.nE; roff = tb.row_off + (size_t)ns.k * tb.nE; rL = tb.row_L;
        Ltot = nfp1(Tab<float>{tb.elE, tb.elL + (size_t)ns.k * tb.nE, tb.nE}, E);
    }
    const float Lneed = Ltot / u;
    int iE = find_monoton(Eg, nE, E);
    if (iE > 1 && fabsf(Eg[iE - 2] - E) < 1.0e-6f) iE -= 1;
    const int o = roff[iE - 1], len = roff[iE] - o;
    const float* L = rL + o;
    float f = 0.f;
    if (len > 1) {
        const int ih = find_decreasing(L, len, Lneed);
        float wf = 0.f;
        if (ih > 1 && ih < len && L[ih - 1] > 0.f && L[ih] > 0.f && L[ih - 1] != L[ih])
            wf = (logf(L[ih - 1]) - logf(Lneed)) / (logf(L[ih - 1]) - logf(L[ih]));
        wf = fminf(fmaxf(wf, 0.f), 0.999f);
        f = ((float)(ih - 1) + wf) / (float)(len - 1);
    }
    X[2 * i] = 2.f * a - 1.f;
    X[2 * i + 1] = prop_u_feature(u);
    Tg[i] = f;
}

// Z += b (per column); H = silu(Z)
__global__ void k_bias_silu(float* Z, const float* __restrict__ b, float* H, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * 64) return;
    const float z = Z[t] + b[t & 63];
    Z[t] = z;
    H[t] = silu(z);
}

// Output layer, loss and the first backward step, one thread per row:
// z2 = Z2 + b2, H2 = silu(z2), y = H2 w3 + b3, dy = 2 (y - t) / n,
// dZ2 = dy w3 silu'(z2); the squared errors are summed into *loss.
__global__ void k_head(const float* __restrict__ Z2, const float* __restrict__ P, const float* __restrict__ Tg, int n,
                       float* H2, float* dZ2, float* DY, float* loss, float* Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float r2 = 0.f;
    if (i < n) {
        const float* b2 = P + OFF_B2;
        const float* w3 = P + OFF_W3;
        float y = P[OFF_B3];
        for (int j = 0; j < 64; ++j) {
            const float z = Z2[(size_t)i * 64 + j] + b2[j], h = silu(z);
            H2[(size_t)i * 64 + j] = h;
            y = fmaf(w3[j], h, y);
        }
        if (Y) Y[i] = y;
        if (Tg) {
            const float r = y - Tg[i], dy = 2.f * r / (float)n;
            r2 = r * r;
            DY[i] = dy;
            for (int j = 0; j < 64; ++j) {
                const float z = Z2[(size_t)i * 64 + j] + b2[j];
                dZ2[(size_t)i * 64 + j] = dy * w3[j] * dsilu(z);
            }
        }
    }
    if (loss) {
        for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        if ((threadIdx.x & 31) == 0 && r2 != 0.f) atomicAdd(loss, r2);
    }
}

// dZ1 = dH1 silu'(Z1)
__global__ void k_back1(const float* __restrict__ dH1, const float* __restrict__ Z1, float* dZ1, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n * 64) dZ1[t] = dH1[t] * dsilu(Z1[t]);
}

__global__ void k_adam(float* P, const float* __restrict__ G, float* m, float* v, int np, float lr, float b1t,
                       float b2t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float g = G[i];
    const float mi = 0.9f * m[i] + 0.1f * g, vi = 0.999f * v[i] + 0.001f * g * g;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi / (1.f - b1t)) / (sqrtf(vi / (1.f - b2t)) + 1e-8f);
}

// Device buffers of one forward/backward pass over at most nmax rows.
struct MlpBufs {
    Buffers b;
    int nmax = 0;
    float *Z1, *H1, *Z2, *H2, *dZ2, *dH1, *dZ1, *DY, *ones, *loss;
    int* err;
    bool alloc(int n) {
        nmax = n;
        const size_t a = (size_t)n * 64;
        Z1 = (float*)b.alloc(4 * a); H1 = (float*)b.alloc(4 * a); Z2 = (float*)b.alloc(4 * a);
        H2 = (float*)b.alloc(4 * a); dZ2 = (float*)b.alloc(4 * a); dH1 = (float*)b.alloc(4 * a);
        dZ1 = (float*)b.alloc(4 * a); DY = (float*)b.alloc(4 * (size_t)n); ones = (float*)b.alloc(16);
        loss = (float*)b.alloc(16); err = (int*)b.alloc(16);
        if (!Z1 || !H1 || !Z2 || !H2 || !dZ2 || !dH1 || !dZ1 || !DY || !ones || !loss || !err) return false;
        const float one = 1.f;
        cudaMemcpy(ones, &one, 4, cudaMemcpyHostToDevice);
        cudaMemset(err, 0, 4);
        return true;
    }
};

static int splits_for(int K) { return std::max(1, std::min(64, K / 256)); }

// Forward pass of n rows (X: n x 2) into H2 and Y; with targets Tg the
// backward pass too, gradients written to G (NP floats).  The four products
// with K = 2, 64 or n run on the tensor cores.
static int mlp_pass(MlpBufs& w, const float* P, const float* X, const float* Tg, int n, float* G, float* Y,
                    cudaStream_t s) {
    const unsigned g64 = (unsigned)((n * 64 + 255) / 256), g1 = (unsigned)((n + 127) / 128);
    int rc = 0;
    // Z1 = X W1, H1 = silu(Z1 + b1)
    rc |= gemm_bf16(X, 2, 1, P + OFF_W1, 64, 1, w.Z1, 64, n, 64, 2, 0, w.err, s);
    k_bias_silu<<<g64, 256, 0, s>>>(w.Z1, P + OFF_B1, w.H1, n);
    // Z2 = H1 W2
    rc |= gemm_bf16(w.H1, 64, 1, P + OFF_W2, 64, 1, w.Z2, 64, n, 64, 64, 0, w.err, s);
    k_head<<<g1, 128, 0, s>>>(w.Z2, P, Tg, n, w.H2, w.dZ2, w.DY, Tg ? w.loss : nullptr, Y);
    if (!Tg) return rc;
    cudaMemsetAsync(G, 0, sizeof(float) * NP, s);
    const int sk = splits_for(n);
    rc |= gemm_bf16(w.H1, 1, 64, w.dZ2, 64, 1, G + OFF_W2, 64, 64, 64, n, 0, w.err, s, sk);   // dW2 = H1^T dZ2
    rc |= gemm_bf16(w.ones, 0, 0, w.dZ2, 64, 1, G + OFF_B2, 64, 1, 64, n, 0, w.err, s, sk);   // db2 = 1^T dZ2
    rc |= gemm_bf16(w.H2, 1, 64, w.DY, 1, 0, G + OFF_W3, 1, 64, 1, n, 0, w.err, s, sk);       // dw3 = H2^T dy
    rc |= gemm_bf16(w.ones, 0, 0, w.DY, 1, 0, G + OFF_B3, 1, 1, 1, n, 0, w.err, s, sk);       // db3 = 1^T dy
    rc |= gemm_bf16(w.dZ2, 64, 1, P + OFF_W2, 1, 64, w.dH1, 64, n, 64, 64, 0, w.err, s);      // dH1 = dZ2 W2^T
    k_back1<<<g64, 256, 0, s>>>(w.dH1, w.Z1, w.dZ1, n);
    rc |= gemm_bf16(X, 1, 2, w.dZ1, 64, 1, G + OFF_W1, 64, 2, 64, n, 0, w.err, s, sk);        // dW1 = X^T dZ1
    rc |= gemm_bf16(w.ones, 0, 0, w.dZ1, 64, 1, G + OFF_B1, 64, 1, 64, n, 0, w.err, s, sk);   // db1 = 1^T dZ1
    return rc;
}

// tensor-core flops of one training pass over n rows (padded tiles not counted)
static double pass_flops(int n) { return 2.0 * n * 64 * (2 + 64) * 3.0 + 2.0 * n * 64 * 3; }

// ---- a trained proposal model attached to a table set ----------------------------------
struct MlpModel {
    Buffers buf;
    MlpDev dev;
    std::vector<NetSpec> specs;
};

static uint16_t to_bf16_bits(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// host copy of the K-major operand offset (bytes) used by the tensor core
static uint32_t kmaj_off_h(int r, int k, int KT) {
    return (uint32_t)((r >> 3) * (KT * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

const MlpDev* mlp_device(const trekis_tables* t) {
    return t->mlp ? &((const MlpModel*)t->mlp.get())->dev : nullptr;
}

// Evaluation of the trained networks: acceptance (the guess is the exact
// bracket), walk length, bisection probes and KL(table || proposal) over the
// bracket histograms of nE energies x nU stratified uniforms per network.
__global__ void k_mlp_eval(DevTabs<float> tb, NetSpec ns, int nEv, int nU, const float* __restrict__ Y,
                           int* __restrict__ exact, int* __restrict__ guessed, int* __restrict__ lens) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nEv * nU) return;
    const int ie = (int)(i / nU), iu = (int)(i % nU);
    const float a = ((float)ie + 0.5f) / (float)nEv, u = ((float)iu + 0.5f) / (float)nU;
    const float E = expf(ns.lo + a * (ns.hi - ns.lo));
    const float* Eg; int nE; const int* roff; const float* rL; float Ltot;
    if (ns.hole) {
        Eg = tb.hE; nE = tb.nH; roff = tb.hrow_off; rL = tb.hrow_L;
        Ltot = nfp1(Tab<float>{tb.hE, tb.hL + (size_t)ns.k * tb.nH, tb.nH}, E);
    } else {
        Eg = tb.elE; nE = tb.nE; roff = tb.row_off + (size_t)ns.k * tb.nE; rL = tb.row_L;
        Ltot = nfp1(Tab<float>{tb.elE, tb.elL + (size_t)ns.k * tb.nE, tb.nE}, E);
    }
    const float Lneed = Ltot / u;
    int iE = find_monoton(Eg, nE, E);
    if (iE > 1 && fabsf(Eg[iE - 2] - E) < 1.0e-6f) iE -= 1;
    const int o = roff[iE - 1], len = roff[iE] - o;
    const float* L = rL + o;
    const int ih = len > 0 ? find_decreasing(L, len, Lneed) : 1;
    const int* mono = ns.hole ? tb.hrow_mono : tb.row_mono + (size_t)ns.k * tb.nE;
    if (!mono[iE - 1]) { exact[i] = 0; guessed[i] = 0; lens[i] = 0; return; }   // the sampler bisects these rows
    const float fg = fminf(fmaxf(Y[i], 0.f), 1.f);
    const int g = 1 + (int)(fg * (float)(len - 1));
    exact[i] = ih;
    guessed[i] = min(max(g, 1), max(len, 1));
    lens[i] = len;
}

// X rows of the evaluation grid (same mapping as k_mlp_eval)
__global__ void k_eval_inputs(int nEv, int nU, float* X) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nEv * nU) return;
    const int ie = (int)(i / nU), iu = (int)(i % nU);
    X[2 * i] = 2.f * (((float)ie + 0.5f) / (float)nEv) - 1.f;
    X[2 * i + 1] = prop_u_feature(((float)iu + 0.5f) / (float)nU);
}

}  // namespace tk

using namespace tk;

extern "C" int32_t trekis_mlp_grad(const float* P, int64_t n, const float* X, const float* Tg, float* grad,
                                   double* loss) {
    if (!P || !X || !Tg || !grad || n <= 0 || n > (1 << 22)) { set_error("invalid arguments"); return TREKIS_EINVAL; }
    MlpBufs w;
    if (!w.alloc((int)n)) return TREKIS_ENOMEM;
    Buffers b;
    float* dP = (float*)b.alloc(4 * NP);
    float* dX = (float*)b.alloc(8 * (size_t)n);
    float* dT = (float*)b.alloc(4 * (size_t)n);
    float* dG = (float*)b.alloc(4 * NP);
    if (!dP || !dX || !dT || !dG) return TREKIS_ENOMEM;
    cudaMemcpy(dP, P, 4 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(dX, X, 8 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(dT, Tg, 4 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemset(w.loss, 0, 4);
    int rc = mlp_pass(w, dP, dX, dT, (int)n, dG, nullptr, 0);
    if (cudaDeviceSynchronize() != cudaSuccess || rc) { set_error("proposal training pass failed"); return TREKIS_ECUDA; }
    int herr = 0;
    float hl = 0.f;
    cudaMemcpy(&herr, w.err, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&hl, w.loss, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(grad, dG, 4 * NP, cudaMemcpyDeviceToHost);
    if (loss) *loss = hl / (double)n;
    if (herr) { set_error("tensor-core wait ran out"); return TREKIS_ETIMEOUT; }
    return TREKIS_OK;
}

extern "C" int32_t trekis_mlp_train(trekis_tables* t, const trekis_mlp_cfg* cfg, trekis_mlp_report* rep) {
    if (!t || !cfg || cfg->n_samples <= 0 || cfg->epochs <= 0 || cfg->batch <= 0 || cfg->batch > (1 << 20) ||
        !(cfg->E_hi > cfg->E_lo) || !(cfg->E_lo > 0)) {
        set_error("invalid proposal training configuration");
        return TREKIS_EINVAL;
    }
    auto* M = new MlpModel();
    std::shared_ptr<void> holder(M, [](void* p) { delete (MlpModel*)p; });
    // one network per electron shell with transfer rows, one for valence holes
    const trekis_material& m = t->mat;
    const int vb = t->shell_index[0][m.atoms[0].N_shl - 1];
    for (int k = 0; k < MAXSH; ++k) M->dev.e_net[k] = -1;
    for (int k = 0; k < t->nsh; ++k) {
        const trekis_atom& at = m.atoms[t->atom_of[k]];
        const double Ip = at.Ip[t->shell_of[k]];
        const double lo = std::log(std::max(cfg->E_lo, Ip + 1.0)), hi = std::log(cfg->E_hi);
        if (!(hi > lo)) continue;
        M->dev.e_net[k] = (int)M->specs.size();
        M->specs.push_back(NetSpec{0, k, (float)lo, (float)hi});
    }
    if (m.hole_mass < 1e3 && t->d32.nH > 0) {
        const double lo = std::log(std::max(cfg->E_lo, m.atoms[0].Ip[m.atoms[0].N_shl - 1] + 1.0));
        const double hi = std::log(std::min(cfg->E_hi, t->Hole_IMFP.E.empty() ? cfg->E_hi : t->Hole_IMFP.E.back()));
        if (hi > lo) {
            M->dev.h_net = (int)M->specs.size();
            M->specs.push_back(NetSpec{1, vb, (float)lo, (float)hi});
        }
    }
    const int nn = (int)M->specs.size();
    if (nn == 0 || nn > MAXNET) { set_error("no network to train"); return TREKIS_EINVAL; }
    M->dev.n_nets = nn;
    for (int q = 0; q < nn; ++q) { M->dev.lo[q] = M->specs[q].lo; M->dev.hi[q] = M->specs[q].hi; }
    float* small = (float*)M->buf.alloc(4 * (size_t)nn * kNetSmall);
    uint16_t* w2t = (uint16_t*)M->buf.alloc(2 * (size_t)nn * 4096);
    if (!small || !w2t) return TREKIS_ENOMEM;
    M->dev.small = small;
    M->dev.w2t = w2t;

    const long long ns = cfg->n_samples;
    const int B = (int)std::min<long long>(cfg->batch, ns);
    MlpBufs w;
    Buffers b;
    if (!w.alloc(B)) return TREKIS_ENOMEM;
    float* X = (float*)b.alloc(8 * (size_t)ns);
    float* Tg = (float*)b.alloc(4 * (size_t)ns);
    float* P = (float*)b.alloc(4 * NP);
    float* G = (float*)b.alloc(4 * NP);
    float* mm = (float*)b.alloc(4 * NP);
    float* vv = (float*)b.alloc(4 * NP);
    const int nEv = std::max(1, cfg->n_eval_E), nU = std::max(2, cfg->n_eval_u);
    const size_t ne = (size_t)nEv * nU;
    float* eX = (float*)b.alloc(8 * ne);
    float* eY = (float*)b.alloc(4 * ne);
    int* eI = (int*)b.alloc(4 * ne);
    int* eG = (int*)b.alloc(4 * ne);
    int* eL = (int*)b.alloc(4 * ne);
    MlpBufs we;
    if (!X || !Tg || !P || !G || !mm || !vv || !eX || !eY || !eI || !eG || !eL || !we.alloc((int)std::min<size_t>(ne, 1 << 20)))
        return TREKIS_ENOMEM;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TREKIS_ECUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    trekis_mlp_report r;
    std::memset(&r, 0, sizeof r);
    r.n_nets = nn;
    double loss_first = 0.0, loss_last = 0.0, flops = 0.0;
    double acc_n = 0.0, acc_ok = 0.0, walk = 0.0, bis = 0.0, kl_sum = 0.0, kl_max = 0.0;
    int kl_n = 0, rc = 0;
    std::vector<float> hp(NP);
    std::vector<float> hsmall((size_t)nn * kNetSmall, 0.f);
    std::vector<uint16_t> hw2((size_t)nn * 4096, 0);
    for (int q = 0; q < nn && !rc; ++q) {
        k_mlp_data<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(t->d32, M->specs[q], cfg->seed, (uint32_t)q, ns, X, Tg);
        // Glorot-normal initial weights, zero biases (host generator keyed by seed and network)
        uint64_t st = cfg->seed * 0x9E3779B97F4A7C15ull + 0x1234567ull * (q + 1);
        auto nrm = [&]() {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const double u1 = ((st >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const double u2 = ((st >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
        };
        std::fill(hp.begin(), hp.end(), 0.f);
        for (int i = 0; i < 128; ++i) hp[OFF_W1 + i] = (float)(nrm() * std::sqrt(2.0 / 66.0));
        for (int i = 0; i < 4096; ++i) hp[OFF_W2 + i] = (float)(nrm() * std::sqrt(2.0 / 128.0));
        for (int i = 0; i < 64; ++i) hp[OFF_W3 + i] = (float)(nrm() * std::sqrt(2.0 / 65.0));
        hp[OFF_B3] = 0.5f;
        cudaMemcpyAsync(P, hp.data(), 4 * NP, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(mm, 0, 4 * NP, s);
        cudaMemsetAsync(vv, 0, 4 * NP, s);
        int step = 0;
        const long long nb = ns / B;
        for (int ep = 0; ep < cfg->epochs && !rc; ++ep) {
            cudaMemsetAsync(w.loss, 0, 4, s);
            const float lr = (float)(cfg->lr * std::pow(0.35, ep));
            for (long long bi = 0; bi < nb && !rc; ++bi) {
                rc |= mlp_pass(w, P, X + 2 * bi * B, Tg + bi * B, B, G, nullptr, s);
                ++step;
                k_adam<<<(NP + 255) / 256, 256, 0, s>>>(P, G, mm, vv, NP, lr, (float)std::pow(0.9, step),
                                                       (float)std::pow(0.999, step));
                flops += pass_flops(B);
                if (ep == 0 && bi == 0) {
                    float l0 = 0.f;
                    cudaMemcpyAsync(&l0, w.loss, 4, cudaMemcpyDeviceToHost, s);
                    cudaStreamSynchronize(s);
                    loss_first += l0 / B / nn;
                    cudaMemsetAsync(w.loss, 0, 4, s);
                }
            }
            if (ep == cfg->epochs - 1) {
                float l1 = 0.f;
                cudaMemcpyAsync(&l1, w.loss, 4, cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
                loss_last += l1 / (double)(nb * B - (cfg->epochs == 1 ? B : 0)) / nn;
            }
        }
        if (cudaGetLastError() != cudaSuccess) rc = -1;
        // evaluation on the stratified grid
        k_eval_inputs<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(nEv, nU, eX);
        for (size_t o = 0; o < ne && !rc; o += (size_t)we.nmax) {
            const int cnt = (int)std::min<size_t>((size_t)we.nmax, ne - o);
            rc |= mlp_pass(we, P, eX + 2 * o, nullptr, cnt, nullptr, eY + o, s);
        }
        k_mlp_eval<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(t->d32, M->specs[q], nEv, nU, eY, eI, eG, eL);
        std::vector<int> hI(ne), hG(ne), hL(ne);
        cudaMemcpyAsync(hI.data(), eI, 4 * ne, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hG.data(), eG, 4 * ne, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hL.data(), eL, 4 * ne, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hp.data(), P, 4 * NP, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = -1;
        for (int ie = 0; ie < nEv && !rc; ++ie) {
            const int len = hL[(size_t)ie * nU];
            if (len < 2) continue;
            std::vector<double> pe(len + 2, 0.0), pg(len + 2, 0.0);
            for (int iu = 0; iu < nU; ++iu) {
                const size_t i = (size_t)ie * nU + iu;
                const int gi = std::min(std::max(hG[i], 1), len), xi = hI[i];
                pe[xi] += 1.0 / nU;
                pg[gi] += 1.0 / nU;
                acc_n += 1.0;
                acc_ok += (gi == xi) ? 1.0 : 0.0;
                walk += std::abs(gi - xi);
                bis += std::ceil(std::log2((double)len));
            }
            double kl = 0.0;
            for (int j = 0; j <= len + 1; ++j)
                if (pe[j] > 0) kl += pe[j] * std::log(pe[j] / std::max(pg[j], 1e-6));
            kl_sum += kl;
            kl_max = std::max(kl_max, kl);
            ++kl_n;
        }
        // inference copy: FP32 small layers, BF16 hidden weights in the operand layout
        float* sm = hsmall.data() + (size_t)q * kNetSmall;
        for (int i = 0; i < 128; ++i) sm[i] = hp[OFF_W1 + i];
        for (int i = 0; i < 64; ++i) { sm[128 + i] = hp[OFF_B1 + i]; sm[192 + i] = hp[OFF_B2 + i]; sm[256 + i] = hp[OFF_W3 + i]; }
        sm[320] = hp[OFF_B3];
        uint16_t* wt = hw2.data() + (size_t)q * 4096;
        for (int i = 0; i < 64; ++i)          // B(k = i, n = j) = W2[i][j]: row j, column i of the operand
            for (int j = 0; j < 64; ++j) wt[kmaj_off_h(j, i, 64) / 2] = to_bf16_bits(hp[OFF_W2 + i * 64 + j]);
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    int herr = 0;
    cudaMemcpy(&herr, w.err, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(small, hsmall.data(), 4 * hsmall.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(w2t, hw2.data(), 2 * hw2.size(), cudaMemcpyHostToDevice);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (rc || cudaDeviceSynchronize() != cudaSuccess) { set_error("proposal training failed"); return TREKIS_ECUDA; }
    if (herr) { set_error("tensor-core wait ran out during training"); return TREKIS_ETIMEOUT; }
    r.train_ms = ms;
    r.tc_gflop = flops * 1e-9;
    r.loss_first = loss_first;
    r.loss_last = loss_last;
    r.kl_mean = kl_n ? kl_sum / kl_n : 0.0;
    r.kl_max = kl_max;
    r.accept_rate = acc_n > 0 ? acc_ok / acc_n : 0.0;
    r.mean_walk = acc_n > 0 ? walk / acc_n : 0.0;
    r.mean_bisect = acc_n > 0 ? bis / acc_n : 0.0;
    if (rep) *rep = r;
    t->mlp = holder;
    return TREKIS_OK;
}

extern "C" int32_t trekis_tc_gemm_bf16(const float* A, int64_t as_m, int64_t as_k, const float* B, int64_t bs_k,
                                       int64_t bs_n, float* C, int64_t ldc, int32_t M, int32_t N, int32_t K,
                                       int32_t accumulate) {
    if (!A || !B || !C || M < 0 || N < 0 || K < 0) { set_error("invalid GEMM arguments"); return TREKIS_EINVAL; }
    int* derr = nullptr;
    if (cudaMalloc(&derr, sizeof(int)) != cudaSuccess) { set_error("cudaMalloc failed"); return TREKIS_ENOMEM; }
    cudaMemset(derr, 0, sizeof(int));
    int rc = gemm_bf16(A, as_m, as_k, B, bs_k, bs_n, C, ldc, M, N, K, accumulate, derr, 0);
    int herr = 0;
    if (cudaDeviceSynchronize() != cudaSuccess || rc) rc = TREKIS_ECUDA;
    cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(derr);
    if (rc) { set_error("tensor-core GEMM launch failed"); return rc; }
    if (herr) { set_error("tensor-core GEMM: bounded MMA wait ran out"); return TREKIS_ETIMEOUT; }
    return TREKIS_OK;
}
