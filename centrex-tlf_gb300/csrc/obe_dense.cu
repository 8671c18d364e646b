// obe_dense.cu -- the dense batched commutator -i[H, rho] on the 5th-generation tensor cores
// (tcgen05.mma, kind::tf32, accumulators in tensor memory), for the measured decision whether a
// dense form beats the sparse gather at >= 64 states.  It is not on the solver's path: the
// measurement (bench.py --case dense76) keeps the sparse gather.
//
// One CTA (four warps) per state.  H and rho (complex, n <= 80, both Hermitian) are split into
// their real and imaginary parts and written to shared memory in the tensor core's K-major,
// unswizzled operand layout: core matrices of 8 rows x 16 bytes, 128 contiguous bytes each; the
// core matrices of one 8-row group follow each other along K at LBO = 2048 bytes, the 8-row groups
// at SBO = 128 bytes.  Every tile is 128 rows (M of one MMA) x 80 columns of K, zero-padded.
//
// With tiles X (row-major) as the A operand and Y as the B operand the MMA computes
// P(X, Y) = X Y^T (B is read K-major).  For Hermitian H and rho, H_re^T = H_re and
// H_im^T = -H_im (likewise rho), so
//   Re(-i[H, rho]) = Im(H rho) - Im(rho H) = -P(Hr,Ri) + P(Hi,Rr) + P(Rr,Hi) - P(Ri,Hr)
//   Im(-i[H, rho]) = Re(rho H) - Re(H rho) = -P(Hr,Rr) - P(Hi,Ri) + P(Rr,Hr) + P(Ri,Hi)
// eight products of ten K-steps (K = 8 per MMA) into two 128 x 80 FP32 accumulators in tensor
// memory (columns 0-79 and 128-207), the signs by the instruction descriptor's negate-A bit.
// Thread 0 issues the 80 MMAs and commits them to an mbarrier; every wait is bounded and reports
// through a status word instead of spinning forever.

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/obe_gb300.h"

namespace {

constexpr int kMaxN = 80;            // N of the MMA (a multiple of 16), and the padded K
constexpr int kRows = 128;           // M of the MMA
constexpr int kLBO = 2048;           // bytes between core matrices along K (16 row groups x 128 B)
constexpr int kSBO = 128;            // bytes between 8-row groups
constexpr int kTileBytes = (kMaxN / 4) * kLBO;  // 20 K-chunks of 4 elements: 40,960 bytes
constexpr int kTiles = 4;            // Hr, Hi, Rr, Ri
// room beyond the four tiles: the mbarrier and the tensor-memory address sit at the end, past any
// address a descriptor of these tiles can reach
constexpr int kSmemBytes = 200 * 1024;
static_assert(kTiles * kTileBytes + 128 <= kSmemBytes, "the tiles and the barrier words must fit");
constexpr int kWaitLimit = 1 << 22;  // mbarrier polls before the CTA gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row r, column k) inside a tile
__device__ __forceinline__ int tile_off(int r, int k) {
    return (k >> 2) * kLBO + (r >> 3) * kSBO + (r & 7) * 16 + (k & 3) * 4;
}

// shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((kLBO >> 4) & 0x3FFF) << 16) |
           (static_cast<uint64_t>((kSBO >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::tf32: D f32, A and B tf32, both K-major, N = 80, M = 128
__host__ __device__ constexpr uint32_t idesc_tf32(bool neg_a) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((neg_a ? 1u : 0u) << 13) | (static_cast<uint32_t>(kMaxN >> 3) << 17) |
           (static_cast<uint32_t>(kRows >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int it = 0; it < kWaitLimit; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// h, rho, out: [count][n][n] complex64 (re, im interleaved); status[0] counts CTAs that gave up
__global__ void __launch_bounds__(128, 1) dense_commutator_kernel(long long count, int n, const float2* __restrict__ h,
                                                                  const float2* __restrict__ rho, float2* __restrict__ out,
                                                                  unsigned int* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* tiles = smem;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kSmemBytes - 128);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kSmemBytes - 64);
    const int tid = static_cast<int>(threadIdx.x), warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(256u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    uint32_t parity = 0;
    bool ok = true;

    for (long long b = blockIdx.x; b < count && ok; b += gridDim.x) {
        const float2* hb = h + static_cast<size_t>(b) * n * n;
        const float2* rb = rho + static_cast<size_t>(b) * n * n;
        // the four tiles, zero outside the n x n block; a warp fills one core matrix at a time
        // (8 rows x 4 columns, 128 contiguous bytes), so its stores meet no bank conflict.  Each
        // thread covers kRows * kMaxN / 128 = 80 elements, in batches of kBatch whose loads are all
        // issued before the first store (four warps per SM leave little else to hide them behind).
        constexpr int kPerThread = kRows * kMaxN / 128, kBatch = 8;
        static_assert(kPerThread % kBatch == 0, "whole batches per thread");
        for (int q0 = 0; q0 < kPerThread; q0 += kBatch) {
            float2 hv[kBatch], rv[kBatch];
            int off[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int q = (q0 + u) * 128 + tid;
                const int t = q & 31, cm = q >> 5;  // core matrix cm = K-chunk * 16 + row group
                const int r = (cm & 15) * 8 + (t >> 2), k = (cm >> 4) * 4 + (t & 3);
                hv[u] = make_float2(0.f, 0.f);
                rv[u] = make_float2(0.f, 0.f);
                if (r < n && k < n) {
                    hv[u] = hb[r * n + k];
                    rv[u] = rb[r * n + k];
                }
                off[u] = tile_off(r, k);
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                *reinterpret_cast<float*>(tiles + 0 * kTileBytes + off[u]) = hv[u].x;
                *reinterpret_cast<float*>(tiles + 1 * kTileBytes + off[u]) = hv[u].y;
                *reinterpret_cast<float*>(tiles + 2 * kTileBytes + off[u]) = rv[u].x;
                *reinterpret_cast<float*>(tiles + 3 * kTileBytes + off[u]) = rv[u].y;
            }
        }
        // generic-proxy writes -> visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t base = smem_u32(tiles);
            // (a tile, b tile, negate) for the real part (accumulator columns 0..79) and the
            // imaginary part (columns 128..207)
            const int terms[2][4][3] = {{{0, 3, 1}, {1, 2, 0}, {2, 1, 0}, {3, 0, 1}},
                                        {{0, 2, 1}, {1, 3, 1}, {2, 0, 0}, {3, 1, 0}}};
            for (int part = 0; part < 2; ++part) {
                const uint32_t d = tmem + static_cast<uint32_t>(part * 128);
                int first = 1;
                for (int t = 0; t < 4; ++t) {
                    const uint32_t a0 = base + terms[part][t][0] * kTileBytes, b0 = base + terms[part][t][1] * kTileBytes;
                    const uint32_t id = idesc_tf32(terms[part][t][2] != 0);
                    for (int ks = 0; ks < kMaxN / 8; ++ks) {
                        mma_tf32(d, smem_desc(a0 + ks * 2 * kLBO), smem_desc(b0 + ks * 2 * kLBO), id, first ? 0u : 1u);
                        first = 0;
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(mbar))
                         : "memory");
        }
        ok = __syncthreads_and(mbar_wait(smem_u32(mbar), parity) ? 1 : 0) != 0;  // one verdict for the CTA
        parity ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (!ok) {
            if (tid == 0) atomicAdd(status, 1u);
            break;
        }
        // epilogue: warp w reads rows 32w..32w+31 (its tensor-memory lanes), 16 columns at a time
        const int row = warp * 32 + lane;
        float2* ob = out + static_cast<size_t>(b) * n * n;
        for (int c0 = 0; c0 < kMaxN; c0 += 16) {
            float re[16], im[16];
            const uint32_t lane_base = tmem + (static_cast<uint32_t>(warp * 32) << 16);
            tmem_ld16(lane_base + static_cast<uint32_t>(c0), re);
            tmem_ld16(lane_base + static_cast<uint32_t>(128 + c0), im);
            if (row < n)
                for (int j = 0; j < 16; ++j)
                    if (c0 + j < n) ob[row * n + c0 + j] = make_float2(re[j], im[j]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();  // tiles and accumulators free for the next state
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(256u) : "memory");
}

}  // namespace

extern "C" obe_status obe_dense_commutator_tf32(int64_t count, int32_t n, const float* d_h, const float* d_rho, float* d_out,
                                                 uint32_t* d_status, void* stream) {
    if (count <= 0 || n <= 0 || n > kMaxN || !d_h || !d_rho || !d_out || !d_status) return OBE_ERR_INVALID;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(dense_commutator_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes) !=
            cudaSuccess)
            return OBE_ERR_CUDA;
        attr = true;
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = count < sms ? count : sms;
    dense_commutator_kernel<<<static_cast<unsigned int>(blocks), 128, kSmemBytes, static_cast<cudaStream_t>(stream)>>>(
        count, n, reinterpret_cast<const float2*>(d_h), reinterpret_cast<const float2*>(d_rho), reinterpret_cast<float2*>(d_out),
        d_status);
    return cudaGetLastError() == cudaSuccess ? OBE_OK : OBE_ERR_CUDA;
}
