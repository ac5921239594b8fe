// Spectral Poisson solve as dense DCT / IDCT / IDXST matrix contractions on the
// 5th-generation tensor cores (tcgen05), in two precisions:
//   * TF32: fp32 operands read as TF32 by kind::tf32, FP32 accumulation;
//   * BF16x3: each operand split into bf16 hi + lo (x = hi + lo to ~16 bits),
//     three products hi.hi + hi.lo + lo.hi per k-step (kind::f16, bf16 inputs),
//     FP32 accumulation.
// The closed forms are those of the FFT path (src/dct2d.rs, src/idct2.rs,
// src/idct_idxst.rs, src/idxst_idct.rs, src/frequencies.rs):
//   A   = (4 / mn) C_m rho C_n^T,   C[k][i] = cos(pi k (2i+1) / 2N)
//   f_x = S_m (W_x . A) D_n^T,  f_y = D_m (W_y . A) S_n^T,  psi = D_m (W_p . A) D_n^T
//   D[i][u] = c_u cos(pi u (2i+1) / 2N), S[i][u] = c_u sin(pi u (2i+1) / 2N), c = (1, 2, 2, ...)
//   W_x = wu / 2k^2, W_y = wv / 2k^2, W_p = 1 / k^2, k^2 = wu^2 + wv^2, [0,0] -> 0.
// Every contraction is written C = A B^T with both operands K-major (row-major,
// K contiguous): the first GEMM of each 2-D transform stores its result
// transposed, which is the K-major operand of the second.
//
// GEMM kernel: one CTA of 128 threads per 128 x BN output tile (BN = 128, or 64
// for the launches with a single contraction, which then fill the SMs).  Thread 0
// issues TMA tile loads (128-byte swizzle) into an S-stage shared-memory ring;
// thread 32 issues the tcgen05.mma instructions into a 128-column FP32
// accumulator (BN columns) in tensor memory and releases each stage with tcgen05.commit; the
// four warps then read the accumulator (tcgen05.ld, one row per thread) and
// store it.  Every mbarrier wait is bounded (status bit kStatusWaitTimeout).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <math.h>

#include <mutex>
#include <vector>

#include "bulk_copy.cuh"
#include "erp_internal.cuh"

namespace erp {

namespace {

constexpr int kTile = 128;   // M and N of an output tile (TMEM lanes x columns)

struct GemmMaps {            // per z: A (hi, lo) and B (hi, lo); lo only for BF16x3
    CUtensorMap a[3][2];
    CUtensorMap b[3][2];
};

struct GemmEpi {
    int mode;                // 0: plain store, 1: weighted spectra (planes)
    int transpose;           // plain: store C^T
    int split;               // store bf16 hi/lo instead of fp32
    int nplanes;             // weighted mode: planes x, y (, p)
    float alpha;             // scale applied before storing
    int ldc;                 // row stride of the stored matrix (elements)
    void *out[3][2];         // per z (plain) or per plane (weighted): fp32 or bf16 hi, bf16 lo
    const float *wu, *wv;    // weighted mode: frequencies of rows (wu) and columns (wv)
    int *status;             // bounded-wait failure flag (kStatusWaitTimeout)
};

// ---- PTX wrappers (tcgen05, TMA) ----
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand tile in shared memory: rows of 128 bytes, 128-byte swizzle
// (as TMA writes it), 8-row groups 1024 bytes apart.  sm_100 descriptor:
// start >> 4 [0,14), leading byte offset >> 4 [16,30) (unused for swizzled
// K-major layouts: 1), stride byte offset >> 4 [32,46), version 1 [46,48),
// layout SWIZZLE_128B = 2 [61,64).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// instruction descriptor: D FP32 [4,6) = 1; A, B format [7,10), [10,13)
// (TF32 = 2 for kind::tf32, BF16 = 1 for kind::f16); K-major A and B; N >> 3
// [17,23); M >> 4 [24,29) (M = 128).
__host__ __device__ constexpr uint32_t instr_desc(uint32_t ab_format, int bn) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(bn >> 3) << 17) |
           ((uint32_t)(kTile >> 4) << 24);
}

template <int KIND, int BN>
__device__ __forceinline__ void mma_issue(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    if (KIND == 0) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(a), "l"(b), "r"(instr_desc(2, BN)), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(a), "l"(b), "r"(instr_desc(1, BN)), "r"(accumulate)
            : "memory");
    }
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Stage ring: A tile 128 x 128 bytes, B tile BN x 128 bytes (+ the lo parts
// for BF16x3).
template <int KIND, int BN>
struct GemmCfg {
    static constexpr int kABytes = kTile * 128, kBBytes = BN * 128;
    static constexpr int kStageBytes = (KIND == 0 ? 1 : 2) * (kABytes + kBBytes);
    // TF32: 3-4 stages (96-99 KB), so two CTAs share an SM and the 128 x 128
    // launches of a 2048^2 solve run in one wave (6 stages: 311 -> 3 stages: 247 us
    // per solve, same bits); BF16 hi/lo stages are twice as large (one CTA per SM)
    static constexpr int kStages = KIND == 0 ? (BN == 128 ? 3 : 4) : (BN == 128 ? 3 : 4);
    static constexpr int kBK = KIND == 0 ? 32 : 64;             // K elements per stage (128 bytes)
    static constexpr size_t kSmem = (size_t)kStages * kStageBytes + 1024;
};

template <int KIND, int BN>
__global__ void __launch_bounds__(128, 1) k_gemm_nt(const __grid_constant__ GemmMaps maps, GemmEpi epi, int K) {
    using Cfg = GemmCfg<KIND, BN>;
    constexpr int S = Cfg::kStages;
    extern __shared__ uint8_t dsm[];
    __shared__ __align__(8) uint64_t full[S], empty[S], done;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(dsm) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int z = blockIdx.z;
    const int tile_m = blockIdx.y * kTile, tile_n = blockIdx.x * BN;
    const int KT = K / Cfg::kBK;

    if (warp == 0) {   // BN accumulator columns; at most two CTAs per SM, so at most 256 of the 512 columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        failed = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    // stage layout: A hi | B hi | A lo | B lo
    auto tile = [&](int s, int op) {
        const size_t off = (op & 1) ? Cfg::kABytes : 0;
        return base + (size_t)s * Cfg::kStageBytes + (size_t)(op >> 1) * (Cfg::kABytes + Cfg::kBBytes) + off;
    };

    if (tid == 0) {   // TMA producer
        for (int kt = 0; kt < KT; ++kt) {
            const int s = kt % S;
            const uint32_t ph = (uint32_t)(kt / S) & 1u;
            if (!mbar_wait(&empty[s], ph ^ 1u)) { failed = 1; break; }
            mbar_expect_tx(&full[s], (uint32_t)Cfg::kStageBytes);
            const int k0 = kt * Cfg::kBK;
            tma_load_2d(tile(s, 0), &maps.a[z][0], k0, tile_m, &full[s]);
            tma_load_2d(tile(s, 1), &maps.b[z][0], k0, tile_n, &full[s]);
            if (KIND == 1) {
                tma_load_2d(tile(s, 2), &maps.a[z][1], k0, tile_m, &full[s]);
                tma_load_2d(tile(s, 3), &maps.b[z][1], k0, tile_n, &full[s]);
            }
        }
    } else if (tid == 32) {   // MMA issuer
        for (int kt = 0; kt < KT; ++kt) {
            const int s = kt % S;
            const uint32_t ph = (uint32_t)(kt / S) & 1u;
            if (!mbar_wait(&full[s], ph)) { failed = 1; break; }
            tc_fence_after();
            const uint32_t a0 = smem_addr(tile(s, 0)), b0 = smem_addr(tile(s, 1));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {   // 4 x 32 bytes of K per 128-byte row
                const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
                if (KIND == 0) {
                    mma_issue<0, BN>(tmem, sw128_desc(a0 + 32 * kk), sw128_desc(b0 + 32 * kk), acc);
                } else {
                    const uint32_t a1 = smem_addr(tile(s, 2)), b1 = smem_addr(tile(s, 3));
                    mma_issue<1, BN>(tmem, sw128_desc(a0 + 32 * kk), sw128_desc(b0 + 32 * kk), acc);   // hi.hi
                    mma_issue<1, BN>(tmem, sw128_desc(a0 + 32 * kk), sw128_desc(b1 + 32 * kk), 1u);    // hi.lo
                    mma_issue<1, BN>(tmem, sw128_desc(a1 + 32 * kk), sw128_desc(b0 + 32 * kk), 1u);    // lo.hi
                }
            }
            mma_commit(&empty[s]);   // the stage is free once these MMAs have read it
        }
        mma_commit(&done);
    }
    __syncwarp();
    const bool ok = mbar_wait(&done, 0u);
    if (!ok && lane == 0) failed = 1;
    tc_fence_after();
    if (ok) {
        // The stage ring is idle now (every MMA has completed): for the weighted
        // spectra and split outputs each warp transposes its 32 x 32 chunks
        // through a 32 x 33 buffer there, so that the many narrow row-major
        // stores go out with consecutive columns across the lanes; plain fp32
        // rows use 128-bit stores of the thread's own row.
        float *buf = reinterpret_cast<float *>(base) + warp * (32 * 33);
        const int r = warp * 32 + lane;   // this thread's accumulator row (TMEM lane)
        const int gr = tile_m + r;
        const float al = epi.alpha;
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (epi.mode == 0 && epi.transpose) {   // C^T: lanes hold consecutive rows already
                if (!epi.split) {
                    float *o = static_cast<float *>(epi.out[z][0]);
#pragma unroll
                    for (int j = 0; j < 32; ++j) o[(size_t)(tile_n + c0 + j) * epi.ldc + gr] = al * v[j];
                } else {
                    __nv_bfloat16 *oh = static_cast<__nv_bfloat16 *>(epi.out[z][0]);
                    __nv_bfloat16 *ol = static_cast<__nv_bfloat16 *>(epi.out[z][1]);
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const size_t idx = (size_t)(tile_n + c0 + j) * epi.ldc + gr;
                        const float x = al * v[j];
                        const __nv_bfloat16 h = __float2bfloat16_rn(x);
                        oh[idx] = h;
                        ol[idx] = __float2bfloat16_rn(x - __bfloat162float(h));
                    }
                }
                continue;
            }
            if (epi.mode == 0 && !epi.split) {   // plain fp32 rows: the thread's 32 columns, 128-bit stores
                float4 *d = reinterpret_cast<float4 *>(static_cast<float *>(epi.out[z][0]) + (size_t)gr * epi.ldc +
                                                       tile_n + c0);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    d[q] = make_float4(al * v[4 * q], al * v[4 * q + 1], al * v[4 * q + 2], al * v[4 * q + 3]);
                continue;
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) buf[lane * 33 + j] = v[j];
            __syncwarp();
            const int gc = tile_n + c0 + lane;
            const float wv = epi.mode == 1 ? epi.wv[gc] : 0.0f;
            const bool three = epi.nplanes > 2;
            for (int rr = 0; rr < 32; ++rr) {
                const int gr2 = tile_m + warp * 32 + rr;
                const size_t idx = (size_t)gr2 * epi.ldc + gc;
                const float x = al * buf[rr * 33 + lane];
                if (epi.mode == 0) {
                    if (!epi.split) {
                        static_cast<float *>(epi.out[z][0])[idx] = x;
                    } else {
                        const __nv_bfloat16 h = __float2bfloat16_rn(x);
                        static_cast<__nv_bfloat16 *>(epi.out[z][0])[idx] = h;
                        static_cast<__nv_bfloat16 *>(epi.out[z][1])[idx] = __float2bfloat16_rn(x - __bfloat162float(h));
                    }
                } else {   // weighted spectra: row u = gr2, column v = gc (planes x, y, p)
                    const float wu = epi.wu[gr2];
                    const float k2 = __fadd_rn(__fmul_rn(wu, wu), __fmul_rn(wv, wv));
                    const float ik = (gr2 == 0 && gc == 0) ? 0.0f : __frcp_rn(k2);
                    const float px = x * (0.5f * wu * ik), py = x * (0.5f * wv * ik), pp = x * ik;
                    if (!epi.split) {
                        static_cast<float *>(epi.out[0][0])[idx] = px;
                        static_cast<float *>(epi.out[1][0])[idx] = py;
                        if (three) static_cast<float *>(epi.out[2][0])[idx] = pp;
                    } else {
                        __nv_bfloat16 h = __float2bfloat16_rn(px);
                        static_cast<__nv_bfloat16 *>(epi.out[0][0])[idx] = h;
                        static_cast<__nv_bfloat16 *>(epi.out[0][1])[idx] = __float2bfloat16_rn(px - __bfloat162float(h));
                        h = __float2bfloat16_rn(py);
                        static_cast<__nv_bfloat16 *>(epi.out[1][0])[idx] = h;
                        static_cast<__nv_bfloat16 *>(epi.out[1][1])[idx] = __float2bfloat16_rn(py - __bfloat162float(h));
                        if (three) {
                            h = __float2bfloat16_rn(pp);
                            static_cast<__nv_bfloat16 *>(epi.out[2][0])[idx] = h;
                            static_cast<__nv_bfloat16 *>(epi.out[2][1])[idx] = __float2bfloat16_rn(pp - __bfloat162float(h));
                        }
                    }
                }
            }
            __syncwarp();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (failed && tid == 0 && epi.status) atomicOr(epi.status, kStatusWaitTimeout);
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
    }
}

__global__ void k_split_bf16(size_t count, const float *__restrict__ src, __nv_bfloat16 *__restrict__ hi,
                             __nv_bfloat16 *__restrict__ lo) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float v = src[i];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

// ---- host side ----
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mu;

bool get_encode() {
    std::lock_guard<std::mutex> lk(g_encode_mu);
    if (g_encode) return true;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return false;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return true;
}

// row-major [rows][cols] matrix, box_rows x 128-byte boxes, 128-byte swizzle
bool make_map(CUtensorMap *map, const void *ptr, int rows, int cols, bool bf16, int box_rows = kTile) {
    const size_t es = bf16 ? 2 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * es};
    cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return g_encode(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                    const_cast<void *>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// A matrix operand: fp32 (TF32) or bf16 hi + lo (BF16x3)
struct GemmOperand {
    void *p[2] = {nullptr, nullptr};
};

struct DctGemmPlan {
    int m = 0, n = 0, kind = 0;   // kind 0: TF32, 1: BF16x3
    cudaStream_t stream = nullptr;
    GemmOperand Cn, Cm, Dn, Sn, Sm, Dm;   // transform matrices
    GemmOperand rho2;                     // BF16x3: split input
    GemmOperand Zt;                       // [n][m] after the first forward contraction
    GemmOperand Aw[3];                    // [m][n] weighted spectra x, y, p
    GemmOperand Zkt[3];                   // [n][m] after the first inverse contraction
    float *wu = nullptr, *wv = nullptr;
    int *status = nullptr;
    int *h_status = nullptr;              // pinned mirror, refreshed after every solve
    std::vector<void *> owned;
    const void *rho_cached = nullptr;     // TF32: the rho the first map was built for
    GemmMaps g1, g2, g3, g4;
};

static bool alloc_operand(DctGemmPlan &P, GemmOperand &o, size_t count) {
    const size_t es = P.kind == 0 ? sizeof(float) : sizeof(__nv_bfloat16);
    for (int h = 0; h < (P.kind == 0 ? 1 : 2); ++h) {
        if (cudaMalloc(&o.p[h], es * count) != cudaSuccess) return false;
        P.owned.push_back(o.p[h]);
    }
    return true;
}

static bool upload_operand(DctGemmPlan &P, GemmOperand &o, const std::vector<double> &v) {
    if (!alloc_operand(P, o, v.size())) return false;
    if (P.kind == 0) {
        std::vector<float> f(v.begin(), v.end());
        return cudaMemcpy(o.p[0], f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    std::vector<__nv_bfloat16> hi(v.size()), lo(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
        const float f = (float)v[i];
        hi[i] = __float2bfloat16_rn(f);
        lo[i] = __float2bfloat16_rn(f - __bfloat162float(hi[i]));
    }
    return cudaMemcpy(o.p[0], hi.data(), 2 * hi.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
           cudaMemcpy(o.p[1], lo.data(), 2 * lo.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

static bool set_maps(const DctGemmPlan &P, CUtensorMap (&dst)[2], const GemmOperand &o, int rows, int cols,
                     int box_rows = kTile) {
    for (int h = 0; h < (P.kind == 0 ? 1 : 2); ++h)
        if (!make_map(&dst[h], o.p[h], rows, cols, P.kind == 1, box_rows)) return false;
    if (P.kind == 0) dst[1] = dst[0];
    return true;
}

void dctgemm_destroy(DctGemmPlan *P) {
    if (!P) return;
    if (P->stream) cudaStreamSynchronize(P->stream);
    for (void *p : P->owned) cudaFree(p);
    if (P->h_status) cudaFreeHost(P->h_status);
    delete P;
}

// transform matrices (FP64 closed forms), buffers and the tensor maps that do
// not depend on the caller's input
DctGemmPlan *dctgemm_create(int m, int n, float bin_w, float bin_h, int kind, cudaStream_t stream,
                            std::string &err) {
    if (m % kTile || n % kTile || m < kTile || n < kTile) {
        err = "the tensor-core solve needs bin counts that are multiples of 128";
        return nullptr;
    }
    if (!get_encode()) {
        err = "cuTensorMapEncodeTiled is not available from the driver";
        return nullptr;
    }
    if (cudaFuncSetAttribute(k_gemm_nt<0, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)GemmCfg<0, 64>::kSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_gemm_nt<0, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)GemmCfg<0, 128>::kSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_gemm_nt<1, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)GemmCfg<1, 64>::kSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_gemm_nt<1, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)GemmCfg<1, 128>::kSmem) != cudaSuccess) {
        err = "cudaFuncSetAttribute failed";
        return nullptr;
    }
    DctGemmPlan *P = new DctGemmPlan();
    P->m = m; P->n = n; P->kind = kind; P->stream = stream;
    const double pi = 3.14159265358979323846;
    auto dct2 = [&](int N) {   // C[k][i] = cos(pi k (2i+1) / 2N)
        std::vector<double> v((size_t)N * N);
        for (int k = 0; k < N; ++k)
            for (int i = 0; i < N; ++i) v[(size_t)k * N + i] = cos(pi * k * (2.0 * i + 1) / (2.0 * N));
        return v;
    };
    auto inv = [&](int N, bool sine) {   // [i][u] = c_u cos|sin(pi u (2i+1) / 2N)
        std::vector<double> v((size_t)N * N);
        for (int i = 0; i < N; ++i)
            for (int u = 0; u < N; ++u) {
                const double a = pi * u * (2.0 * i + 1) / (2.0 * N), c = u == 0 ? 1.0 : 2.0;
                v[(size_t)i * N + u] = c * (sine ? sin(a) : cos(a));
            }
        return v;
    };
    const size_t mn = (size_t)m * n;
    bool ok = upload_operand(*P, P->Cn, dct2(n)) && upload_operand(*P, P->Cm, dct2(m)) &&
              upload_operand(*P, P->Dn, inv(n, false)) && upload_operand(*P, P->Sn, inv(n, true)) &&
              upload_operand(*P, P->Sm, inv(m, true)) && upload_operand(*P, P->Dm, inv(m, false)) &&
              alloc_operand(*P, P->Zt, mn);
    for (int k = 0; ok && k < 3; ++k) ok = alloc_operand(*P, P->Aw[k], mn) && alloc_operand(*P, P->Zkt[k], mn);
    if (ok && kind == 1) ok = alloc_operand(*P, P->rho2, mn);
    std::vector<float> hu(m), hv(n);   // frequencies as the FFT path builds them
    const float tpm = (float)(2.0 * pi) / (float)m, tpn = (float)(2.0 * pi) / (float)n, wv_div = bin_w / bin_h;
    for (int i = 0; i < m; ++i) hu[i] = (float)i * tpm;
    for (int j = 0; j < n; ++j) hv[j] = ((float)j * tpn) * wv_div;
    ok = ok && cudaMalloc(&P->wu, sizeof(float) * m) == cudaSuccess;
    if (ok) P->owned.push_back(P->wu);
    ok = ok && cudaMalloc(&P->wv, sizeof(float) * n) == cudaSuccess;
    if (ok) P->owned.push_back(P->wv);
    ok = ok && cudaMalloc(&P->status, sizeof(int)) == cudaSuccess;
    if (ok) P->owned.push_back(P->status);
    ok = ok && cudaMallocHost((void **)&P->h_status, sizeof(int)) == cudaSuccess;
    if (ok) *P->h_status = 0;
    ok = ok && cudaMemcpy(P->wu, hu.data(), sizeof(float) * m, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->wv, hv.data(), sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(P->status, 0, sizeof(int)) == cudaSuccess;
    // maps: G1 A = rho (per call for TF32, rho2 for BF16x3), B = C_n;  G2 A = C_m, B = Zt;
    // G3 A = Aw[k], B = D_n / S_n / D_n;  G4 A = S_m / D_m / D_m, B = Zkt[k]
    // G1 and G2 (one contraction per launch) use 128 x 64 tiles: twice the CTAs
    ok = ok && set_maps(*P, P->g1.b[0], P->Cn, n, n, 64) && set_maps(*P, P->g2.a[0], P->Cm, m, m) &&
         set_maps(*P, P->g2.b[0], P->Zt, n, m, 64);
    if (ok && kind == 1) ok = set_maps(*P, P->g1.a[0], P->rho2, m, n);
    const GemmOperand *b3[3] = {&P->Dn, &P->Sn, &P->Dn}, *a4[3] = {&P->Sm, &P->Dm, &P->Dm};
    for (int k = 0; ok && k < 3; ++k)
        ok = set_maps(*P, P->g3.a[k], P->Aw[k], m, n) && set_maps(*P, P->g3.b[k], *b3[k], n, n) &&
             set_maps(*P, P->g4.a[k], *a4[k], m, m) && set_maps(*P, P->g4.b[k], P->Zkt[k], n, m);
    if (!ok) {
        err = "tensor-core solve set-up failed";
        dctgemm_destroy(P);
        return nullptr;
    }
    return P;
}

template <int KIND, int BN>
static cudaError_t launch_gemm(const DctGemmPlan &P, const GemmMaps &maps, const GemmEpi &epi, int M, int N,
                               int K, int Z) {
    dim3 grid(N / BN, M / kTile, Z);
    k_gemm_nt<KIND, BN><<<grid, 128, GemmCfg<KIND, BN>::kSmem, P.stream>>>(maps, epi, K);
    return cudaGetLastError();
}

static cudaError_t run_gemm(const DctGemmPlan &P, const GemmMaps &maps, const GemmEpi &epi, int M, int N, int K,
                            int Z, int bn) {
    if (bn == 64)
        return P.kind == 0 ? launch_gemm<0, 64>(P, maps, epi, M, N, K, Z) : launch_gemm<1, 64>(P, maps, epi, M, N, K, Z);
    return P.kind == 0 ? launch_gemm<0, 128>(P, maps, epi, M, N, K, Z)
                       : launch_gemm<1, 128>(P, maps, epi, M, N, K, Z);
}

// fx, fy (, psi) = Poisson solve of rho: four contraction launches (+ the split
// of rho).  Returns cudaErrorTimeout when a bounded wait of an earlier solve
// on this plan ran out (seen through the pinned mirror of the status word).
//
// status: where the contractions report a bounded wait that ran out; nullptr
// uses the plan's own word and its pinned mirror (a placement context passes
// its DevState status, read by the host with the rest of the state).
cudaError_t dctgemm_solve(DctGemmPlan &P, const float *rho, float *fx, float *fy, float *psi, int *status) {
    if (!status && *(volatile int *)P.h_status) return cudaErrorTimeout;
    const int m = P.m, n = P.n, nk = psi ? 3 : 2;
    const size_t mn = (size_t)m * n;
    const bool split = P.kind == 1;
    cudaError_t e = cudaSuccess;
    if (split) {
        k_split_bf16<<<152 * 8, 256, 0, P.stream>>>(mn, rho, (__nv_bfloat16 *)P.rho2.p[0],
                                                   (__nv_bfloat16 *)P.rho2.p[1]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    } else if (rho != P.rho_cached) {
        if (!make_map(&P.g1.a[0][0], rho, m, n, false)) return cudaErrorInvalidValue;
        P.g1.a[0][1] = P.g1.a[0][0];
        P.rho_cached = rho;
    }
    GemmEpi ep;
    memset(&ep, 0, sizeof ep);
    ep.status = status ? status : P.status;
    ep.split = split ? 1 : 0;
    // G1: Z = rho C_n^T, stored transposed [n][m]
    ep.mode = 0; ep.transpose = 1; ep.alpha = 1.0f; ep.ldc = m;
    ep.out[0][0] = P.Zt.p[0]; ep.out[0][1] = P.Zt.p[1];
    if ((e = run_gemm(P, P.g1, ep, m, n, n, 1, 64)) != cudaSuccess) return e;
    // G2: A = (4/mn) C_m Z, written as the weighted spectra [m][n]
    ep.mode = 1; ep.transpose = 0; ep.alpha = (float)(4.0 / ((double)m * (double)n)); ep.ldc = n;
    ep.nplanes = nk; ep.wu = P.wu; ep.wv = P.wv;
    for (int k = 0; k < 3; ++k) { ep.out[k][0] = P.Aw[k].p[0]; ep.out[k][1] = P.Aw[k].p[1]; }
    if ((e = run_gemm(P, P.g2, ep, m, n, m, 1, 64)) != cudaSuccess) return e;
    // G3: Z_k = Aw_k (D_n | S_n | D_n)^T, stored transposed [n][m]
    ep.mode = 0; ep.transpose = 1; ep.alpha = 1.0f; ep.ldc = m; ep.nplanes = 0;
    for (int k = 0; k < 3; ++k) { ep.out[k][0] = P.Zkt[k].p[0]; ep.out[k][1] = P.Zkt[k].p[1]; }
    if ((e = run_gemm(P, P.g3, ep, m, n, n, nk, 128)) != cudaSuccess) return e;
    // G4: field_x = S_m Z_x, field_y = D_m Z_y, psi = D_m Z_p, fp32 [m][n]
    ep.split = 0; ep.transpose = 0; ep.ldc = n;
    float *outs[3] = {fx, fy, psi};
    for (int k = 0; k < 3; ++k) { ep.out[k][0] = outs[k]; ep.out[k][1] = nullptr; }
    if ((e = run_gemm(P, P.g4, ep, m, n, m, nk, 128)) != cudaSuccess) return e;
    if (status) return cudaSuccess;
    return cudaMemcpyAsync(P.h_status, P.status, sizeof(int), cudaMemcpyDeviceToHost, P.stream);
}

}  // namespace erp
