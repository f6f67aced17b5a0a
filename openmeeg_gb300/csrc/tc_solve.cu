// Persistent triangular sweep of the mixed-precision solver (sm_103a, tcgen05).
//
// The FP32 factor HM = L diag(+I, -I) L^T is stored with the diagonal-block
// inverses folded into the solve operators (W_j = L21_j Linv_j for the forward
// sweep, Linv_j L_j,: block rows for the backward one), so a sweep is
//
//   forward:   x~_k = b_k - sum_{j<k} W_j[block k rows] x~_j
//   backward:  x~_k = y_k - sum_{j>k} (Linv_j L_jk)^T x~_j
//
// over 128-row blocks k, followed by one launch that applies the inverses to
// every block.  One launch does the whole sweep: CTAs claim output tiles
// (block k x 64 right-hand sides) in dependency order from a global counter;
// a tile accumulates its products in TMEM as soon as the blocks it needs are
// published, then publishes the TF32 head/remainder split of x~_k (the operand
// of later tiles) with a release flag, and writes x~_k into B.  Tiles are
// claimed in increasing order and a tile depends only on smaller ones, so the
// smallest unfinished tile can always proceed: no co-residency of the CTAs is
// assumed.
//
// Per CTA: warp 0 waits (acquire) for block j's flag, then streams the four
// 32-deep K chunks of the operator block (128 x 32, head + remainder) and of
// the published split (64 x 32, head + remainder) into a four-stage ring with
// TMA (128-byte swizzle); warp 1 issues tcgen05.mma.kind::tf32 (M = 128,
// N = 64, K = 8; 3xTF32: hh + hl + lh) into a 64-column TMEM accumulator;
// warps 2-9 load their b_k values while the products run, read the
// accumulator (tcgen05.ld), publish the split and store x~_k.  The dependency
// chain is the sweep's critical path: per block a flag hand-over, one block
// product and the epilogue (about 5 us on a GB300).  Every wait is bounded: on
// timeout the kernel records OMG_ERR_TIMEOUT, stops, lets its copies in flight
// land (bounded), releases TMEM and returns; CTAs waiting on its tiles time out
// in turn.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "device_common.cuh"
#include "omg_internal.h"
#include "tcgen05.cuh"

namespace omg {
namespace tcs {

using namespace tc;

constexpr int BM = 128;                           // rows of a block (TMEM lanes)
constexpr int BN = 64;                            // right-hand sides of a tile (TMEM columns)
constexpr int BK = 32;                            // K per chunk (128 bytes of FP32: one swizzle atom)
constexpr int KB = 128;                           // K of one block product
constexpr int NCHUNK = KB / BK;
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * BK * 4;              // 16 KiB
constexpr int B_BYTES = BN * BK * 4;              // 8 KiB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
constexpr int THREADS = 320;                      // producer, MMA, 8 epilogue warps
constexpr int EC = BN / 2;                        // columns per epilogue thread (two warps per lane quarter)
constexpr uint32_t TMEM_COLS = BN;
constexpr uint32_t FLAG_POLLS = 1u << 22;         // bounded wait on another tile (~seconds)

// D = F32, A = B = TF32, both K-major, N = BN, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Orders this thread's generic-proxy global accesses with async-proxy (TMA) ones.
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

struct SweepArgs {
    int backward;        // 0: forward sweep (W operators), 1: backward sweep (folded block rows of the factor)
    int nblocks;         // 128-row blocks (the last may be shorter)
    int N;               // rows of B
    int nrhs;            // right-hand sides
    int ncg;             // groups of BN right-hand sides
    int ncolpad;         // ncg * BN
    float* B;            // N x nrhs, column-major, leading dimension ldb (x~ on return)
    int64_t ldb;
    float* XSh;          // published split of block k, group cg: rows k * ncolpad + cg * BN .., 128 floats each
    float* XSl;
    int* flags;          // nblocks * ncg, 1 once the tile's split is published
    int* counter;        // tile claims
    int* err;
};

__global__ void __launch_bounds__(THREADS, 1)
    sweep_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                 const __grid_constant__ CUtensorMap tXh, const __grid_constant__ CUtensorMap tXl, const SweepArgs a) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], tfull_bar, fin_bar;
    __shared__ uint32_t tmem_holder;
    __shared__ volatile int s_abort;
    __shared__ int s_tile;
    __shared__ int64_t s_issued, s_consumed;
    const uint32_t sbase = (dev::smem_u32(smem_raw) + 1023u) & ~1023u;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int ntiles = a.nblocks * a.ncg;
    if (threadIdx.x == 0) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tAh)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tXh)) : "memory");
        for (int s = 0; s < STAGES; ++s) {
            dev::mbar_init(&full_bar[s], 1);
            dev::mbar_init(&empty_bar[s], 1);
        }
        dev::mbar_init(&tfull_bar, 1);
        dev::mbar_init(&fin_bar, 1);
        s_abort = 0;
        s_issued = 0;
        s_consumed = 0;
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         dev::smem_u32(&tmem_holder)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_holder;
    int64_t g_prod = 0, g_mma = 0;   // chunk counters of the producer and the MMA issuer (same sequence)
    bool issued_any = false;         // MMA issuer: some product was issued by this CTA
    uint32_t lt = 0;                 // tiles done by this CTA (accumulator phase)

    for (;;) {
        if (threadIdx.x == 0) s_tile = s_abort ? ntiles : atomicAdd(a.counter, 1);
        __syncthreads();
        const int t = s_tile;
        if (t >= ntiles || s_abort) break;
        const int kq = t / a.ncg, cg = t % a.ncg;
        const int k = a.backward ? a.nblocks - 1 - kq : kq;
        const int nj = a.backward ? a.nblocks - 1 - k : k;     // blocks this tile takes products from
        const int k0 = k * BM;

        if (warp == 0) {
            if (lane == 0) {   // ---- producer
                for (int i = 0; i < nj && !s_abort; ++i) {
                    const int j = a.backward ? a.nblocks - 1 - i : i;
                    for (int c = 0; c < NCHUNK; ++c, ++g_prod) {
                        const int slot = (int)(g_prod % STAGES);
                        if (!wait_or_abort(&empty_bar[slot], (uint32_t)(((g_prod / STAGES) & 1) ^ 1), &s_abort)) {
                            s_abort = 1;
                            break;
                        }
                        if (c == 0) {   // block j of this column group must be published
                            const int* f = a.flags + (int64_t)j * a.ncg + cg;
                            uint32_t it = 0;
                            while (ld_acquire(f) == 0 && !s_abort && ++it < FLAG_POLLS) __nanosleep(64);
                            if (it >= FLAG_POLLS || s_abort) {
                                s_abort = 1;
                                break;
                            }
                            fence_proxy_async_global();
                        }
                        const uint32_t st = sbase + slot * STAGE_BYTES;
                        dev::mbar_expect_tx(&full_bar[slot], STAGE_BYTES);
                        int ya, yr, xa;
                        if (a.backward) {
                            xa = j * BM + c * BK;
                            ya = yr = k0;
                        } else {
                            const int k1j = (j + 1) * BM;
                            xa = c * BK;
                            // W_j's heads start at K-major row 2 j N - 128 j (j + 1) (each W_b holds the
                            // N - k1_b rows below block b, heads then remainders)
                            ya = (int)(2 * (int64_t)j * a.N - 128 * (int64_t)j * (j + 1)) + (k0 - k1j);
                            yr = ya + (a.N - k1j);
                        }
                        tma_load_2d(st, &tAh, xa, ya, &full_bar[slot]);
                        tma_load_2d(st + A_BYTES, a.backward ? &tAl : &tAh, xa, yr, &full_bar[slot]);
                        const int yx = j * a.ncolpad + cg * BN;
                        tma_load_2d(st + 2 * A_BYTES, &tXh, c * BK, yx, &full_bar[slot]);
                        tma_load_2d(st + 2 * A_BYTES + B_BYTES, &tXl, c * BK, yx, &full_bar[slot]);
                        s_issued = g_prod + 1;
                    }
                    if (s_abort) break;
                }
            }
        } else if (warp == 1) {
            if (lane == 0) {   // ---- MMA issuer
                bool ok = true;
                for (int i = 0; i < nj && ok; ++i) {
                    for (int c = 0; c < NCHUNK; ++c, ++g_mma) {
                        const int slot = (int)(g_mma % STAGES);
                        if (!wait_or_abort(&full_bar[slot], (uint32_t)((g_mma / STAGES) & 1), &s_abort)) {
                            ok = false;
                            break;
                        }
                        s_consumed = g_mma + 1;
                        fence_after();
                        const uint32_t st = sbase + slot * STAGE_BYTES;
                        const uint64_t dAh = sdesc_sw128(st), dAl = sdesc_sw128(st + A_BYTES);
                        const uint64_t dXh = sdesc_sw128(st + 2 * A_BYTES);
                        const uint64_t dXl = sdesc_sw128(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
                        for (int kk = 0; kk < BK / 8; ++kk) {
                            const uint64_t off = (uint64_t)(kk * 32) >> 4;
                            mma_tf32(tmem, dAh + off, dXh + off, (i | c | kk) != 0 ? 1u : 0u);
                            mma_tf32(tmem, dAh + off, dXl + off, 1u);
                            mma_tf32(tmem, dAl + off, dXh + off, 1u);
                        }
                        mma_commit(&empty_bar[slot]);
                        issued_any = true;
                    }
                }
                if (!ok) s_abort = 1;
                if (nj > 0)
                    mma_commit(&tfull_bar);   // the accumulator is complete once these products are done
                else
                    mbar_arrive(&tfull_bar);  // nothing to accumulate
            }
        } else {   // ---- epilogue: TMEM lanes 32 * (warp % 4) .. +31, EC of the BN columns
            const int q = warp & 3;
            const int half = (warp - 2) / 4;
            const int r = k0 + q * 32 + lane;                 // row of B
            const int rl = q * 32 + lane;                     // row within the block (K of later products)
            const int cb = cg * BN + half * EC;               // first right-hand side of this thread
            float* __restrict__ const bp = a.B + r + (int64_t)cb * a.ldb;
            // this thread's values of b_k, loaded while the products run (independent of them)
            const int ncol = r < a.N ? min(EC, a.nrhs - cb) : 0;
            float bv[EC];
#pragma unroll
            for (int u = 0; u < EC; ++u) bv[u] = u < ncol ? __ldcg(bp + (int64_t)u * a.ldb) : 0.f;
            bool ok = wait_or_abort(&tfull_bar, lt & 1u, &s_abort);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                if (lane == 0) s_abort = 1;
            } else {
                fence_after();
                float* __restrict__ const xh = a.XSh + ((int64_t)k * a.ncolpad + cb) * KB + rl;
                float* __restrict__ const xl = a.XSl + ((int64_t)k * a.ncolpad + cb) * KB + rl;
                const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * EC);
                uint32_t v[EC];
                if (nj > 0) {
                    tmem_ld32(tb, v);
                } else {
#pragma unroll
                    for (int u = 0; u < EC; ++u) v[u] = 0u;
                }
                // x~ replaces the prefetched values; its split is published first
#pragma unroll
                for (int u = 0; u < EC; ++u) {
                    const float x = bv[u] - __uint_as_float(v[u]);
                    const float h = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
                    __stcg(xh + (int64_t)u * KB, h);
                    __stcg(xl + (int64_t)u * KB, x - h);
                    bv[u] = x;
                }
            }
            // publish the split: every epilogue thread's stores, then one release of the flag
            fence_proxy_async_global();
            __threadfence();
            asm volatile("bar.sync 1, 256;" ::: "memory");
            if (warp == 2 && lane == 0 && !s_abort) st_release(a.flags + (int64_t)k * a.ncg + cg, 1);
            // then x~ into B (read only after the sweep)
            if (ok) {
#pragma unroll
                for (int u = 0; u < EC; ++u)
                    if (u < ncol) __stcg(bp + (int64_t)u * a.ldb, bv[u]);
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
        ++lt;
    }

    // ---- shutdown: products and copies in flight complete before TMEM goes
    if (warp == 1 && lane == 0) {
        if (issued_any)
            mma_commit(&fin_bar);
        else
            mbar_arrive(&fin_bar);
        if (!dev::mbar_wait_bounded(&fin_bar, 0)) s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
        if (threadIdx.x == 0) {
            atomicExch(a.err, -8 /* OMG_ERR_TIMEOUT */);
            for (int64_t g = s_consumed; g < s_issued; ++g)
                dev::mbar_wait_bounded(&full_bar[g % STAGES], (uint32_t)((g / STAGES) & 1));
        }
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

static_assert(EC == 32, "one 32-column TMEM load per epilogue thread");
static_assert(STAGES * STAGE_BYTES + 1024 <= 227 * 1024, "shared memory");

}  // namespace tcs

static inline void check_tcs(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}

static int64_t sweep_ncolpad(int64_t nrhs) { return (nrhs + tcs::BN - 1) / tcs::BN * tcs::BN; }

// Scratch of the persistent sweeps of one solve: published splits and flags.
size_t sweep_scratch_bytes(int64_t nblocks, int64_t nrhs) {
    const int64_t ncolpad = sweep_ncolpad(nrhs), ncg = ncolpad / tcs::BN;
    return (size_t)2 * nblocks * ncolpad * tcs::KB * 4 + (size_t)(nblocks * ncg + 32) * 4;
}

// One triangular sweep (see the file comment).  Forward: operators W (rows of
// 128 floats; W_j's heads start at row 2 j N - 128 j (j + 1), its remainders
// N - k1_j rows later; w_rows rows in all).  Backward: heads A and remainders
// Ar of the factor (column-major, leading dimension ld).  B: N x nrhs FP32,
// column-major.  `scratch` holds sweep_scratch_bytes(nblocks, nrhs) bytes.
void solve_sweep_tc(bool backward, int64_t N, int64_t nblocks, const float* W, int64_t w_rows, const float* A,
                    const float* Ar, int64_t ld, float* B, int64_t ldb, int64_t nrhs, void* scratch, int* err,
                    cudaStream_t s, int max_ctas) {
    if (nrhs <= 0 || N <= 0) return;
    if (N > (int64_t)INT32_MAX / 2 || nblocks * tcs::BM < N || (nblocks - 1) * tcs::BM >= N)
        throw Error(OMG_ERR_INVALID, "solve sweep: blocks do not cover the rows");
    if (!backward && 2 * (nblocks - 1) * N > (int64_t)INT32_MAX)
        throw Error(OMG_ERR_UNSUPPORTED, "solve sweep: operator rows beyond 32-bit TMA coordinates");
    ProfScope prof_("solve_sweep", s);
    const int64_t ncolpad = sweep_ncolpad(nrhs), ncg = ncolpad / tcs::BN;
    if (nblocks * ncolpad > (int64_t)INT32_MAX) throw Error(OMG_ERR_UNSUPPORTED, "solve sweep: too many columns");
    float* XSh = static_cast<float*>(scratch);
    float* XSl = XSh + nblocks * ncolpad * tcs::KB;
    int* flags = reinterpret_cast<int*>(XSl + nblocks * ncolpad * tcs::KB);
    int* counter = flags + nblocks * ncg;
    OMG_CUDA(cudaMemsetAsync(flags, 0, (size_t)(nblocks * ncg + 1) * 4, s));
    CUtensorMap mAh, mAl;
    if (backward) {
        mAh = tc::make_map_2d(A, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, N, N, ld, tcs::BK, tcs::BM);
        mAl = tc::make_map_2d(Ar, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, N, N, ld, tcs::BK, tcs::BM);
    } else {
        mAh = tc::make_map_2d(W, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, w_rows, tcs::KB, tcs::KB, tcs::BK, tcs::BM);
        mAl = mAh;
    }
    const CUtensorMap mXh =
        tc::make_map_2d(XSh, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nblocks * ncolpad, tcs::KB, tcs::KB, tcs::BK, tcs::BN);
    const CUtensorMap mXl =
        tc::make_map_2d(XSl, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nblocks * ncolpad, tcs::KB, tcs::KB, tcs::BK, tcs::BN);
    static bool attr = false;
    static int n_sm = 0;
    if (!attr) {
        cudaFuncSetAttribute(tcs::sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tcs::SMEM_BYTES);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (n_sm <= 0) n_sm = 1;
        attr = true;
    }
    tcs::SweepArgs args{backward ? 1 : 0, (int)nblocks, (int)N, (int)nrhs, (int)ncg, (int)ncolpad, B, ldb, XSh, XSl,
                        flags, counter, err};
    // max_ctas > 0 leaves SMs to work on another stream: most CTAs of a sweep wait on the block chain
    const int cap = max_ctas > 0 ? std::min(max_ctas, n_sm) : n_sm;
    const unsigned grid = (unsigned)std::min<int64_t>(nblocks * ncg, cap);
    tcs::sweep_kernel<<<grid, tcs::THREADS, tcs::SMEM_BYTES, s>>>(mAh, mAl, mXh, mXl, args);
    check_tcs("solve sweep");
}

}  // namespace omg
