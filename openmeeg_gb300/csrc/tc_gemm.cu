// Tensor-core GEMM for the mixed-precision solver (sm_103a, tcgen05).
//
//   C = beta * C + alpha * A * B^T          A: M x K, B: N x K (both K-major)
//
// FP32 accuracy on the TF32 tensor pipe by operand splitting: each FP32
// operand is X = Xh + Xl with Xh the TF32-representable head (low 13
// mantissa bits cleared) and Xl = X - Xh; the product is accumulated as
// Ah*Bh + Ah*Bl + Al*Bh (the "3xTF32" scheme), with FP32 accumulation in TMEM.
//
// Persistent and warp-specialized: one CTA per SM walks a static list of
// 128 x 128 output tiles (all tiles, or the lower triangle for a symmetric
// update).  Warp 0 streams the K dimension in 32-element (128-byte) chunks
// into a three-stage shared-memory ring with TMA (cp.async.bulk.tensor,
// 128-byte swizzle); warp 1 issues tcgen05.mma.cta_group::1.kind::tf32
// (M=128, N=128, K=8) into one of two TMEM accumulators, so the next tile's
// products overlap the previous tile's epilogue; warps 2-9 (two per TMEM lane
// quarter, 64 columns each) load the tile's C into registers while its
// products run, then read their TMEM lanes with tcgen05.ld and write C.  Stages and accumulators are handed over with
// mbarriers (TMA complete_tx, tcgen05.commit, epilogue arrivals).  Every wait
// is bounded: on timeout the kernel records OMG_ERR_TIMEOUT, every role stops,
// copies and products in flight are waited for (bounded), TMEM is released
// and the CTA returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <climits>
#include <memory>
#include <mutex>
#include <vector>

#include "device_common.cuh"
#include "omg_internal.h"
#include "tcgen05.cuh"

namespace omg {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 4;           // 16 KiB (BM == BN)
constexpr int STAGE_BYTES = 4 * TILE_BYTES;       // Ah, Al, Bh, Bl
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
constexpr int THREADS = 320;                      // producer, MMA, 8 epilogue warps
constexpr int EPI_WARPS = 8;                      // two per TMEM lane quarter, 64 columns each
constexpr uint32_t TMEM_COLS = 256;               // two 128-column FP32 accumulators

// Instruction descriptor: D=F32, A=B=TF32, both K-major, N=128, M=128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

// Tile t of the walk -> (tile row, tile column).  Lower: row-major over the
// lower triangle (diagonal included); otherwise column of tiles after column.
__device__ __forceinline__ void tile_of(int64_t t, int tiles_m, int lower, int& tm, int& tn) {
    if (lower) {
        int r = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);   // FP32 guess, corrected exactly below
        while ((int64_t)r * (r + 1) / 2 > t) --r;
        while ((int64_t)(r + 1) * (r + 2) / 2 <= t) ++r;
        tm = r;
        tn = (int)(t - (int64_t)r * (r + 1) / 2);
    } else {
        tm = (int)(t % tiles_m);
        tn = (int)(t / tiles_m);
    }
}

// Optional epilogue outputs besides C (null pointers: off).
//  Sh/Sl  K-major TF32 head / remainder copy of C's rows >= s_row0: row i of C
//         becomes row i - s_row0 (row stride s_kpad), zero past column N.
//  Cr     C receives the TF32 head of each value and Cr (same layout) the
//         remainder (beta must be 0).
//  Xh/Xl  K-major head / remainder copy of the 128-row band of C starting at
//         row x_row0 (a multiple of 128), transposed: column j of the band
//         becomes row j (stride 128), rows past M written as zero.
struct EpiArgs {
    float* Sh;
    float* Sl;
    float* Cr;
    float* Xh;
    float* Xl;
    int s_row0, s_kpad, x_row0;
};

// Grouped launch: independent products C_p (M_p x N_p, ldc_p) = alpha A_p B_p^T,
// written as TF32 heads (C_p) and remainders (Cr_p), walked as one list of
// tiles by one persistent launch.  The operand tiles of product p are read
// through the first (set 0) or second (set 1) group of tensor maps at row
// coordinates ay_h / ay_l (A heads / remainders, + 128 tm) and by_h / by_l
// (B, + 128 tn), K coordinates ax / bx (+ 32 per chunk).  Rows past M_p or N_p
// read whatever the map holds there (zero past its extent); they only feed
// accumulator rows and columns that are not written.
constexpr int MAX_GROUP = 320;
struct GroupEntry {
    float* C;
    float* Cr;
    int ldc, M, N, K, set;
    int ay_h, ay_l, by_h, by_l, ax, bx;
    int tile0;   // first tile of this product in the walk
};
template <bool G>
struct GroupParam {   // empty for the single-product kernel
    int n;
};
template <>
struct GroupParam<true> {
    int n;
    GroupEntry g[MAX_GROUP];
};

// The tile a role works on: position, K chunks, output.
struct TileJob {
    int tm, tn, nk, M, N, ldc, p;
    float* C;
    float* Cr;
};

template <bool G>
__device__ __forceinline__ TileJob tile_job(int64_t t, const GroupParam<G>& gp, int tiles_m, int lower, int M, int N,
                                            int nk, float* C, int64_t ldc, float* Cr) {
    TileJob j;
    if constexpr (G) {
        int lo = 0, hi = gp.n - 1;   // last product whose first tile is <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (gp.g[mid].tile0 <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        const GroupEntry& e = gp.g[lo];
        const int tmz = (e.M + BM - 1) / BM, loc = (int)(t - e.tile0);
        j.tm = loc % tmz;
        j.tn = loc / tmz;
        j.nk = (e.K + BK - 1) / BK;
        j.M = e.M;
        j.N = e.N;
        j.ldc = e.ldc;
        j.C = e.C;
        j.Cr = e.Cr;
        j.p = lo;
    } else {
        tile_of(t, tiles_m, lower, j.tm, j.tn);
        j.nk = nk;
        j.M = M;
        j.N = N;
        j.ldc = (int)ldc;
        j.C = C;
        j.Cr = Cr;
        j.p = 0;
    }
    return j;
}

// K may come in two segments with their own operand maps (the second set is
// used for the chunks past K0 when K > K0): an update by two panels at once.
template <bool G>
__global__ void __launch_bounds__(THREADS, 1)
    gemm_tf32x3_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                       const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl,
                       const __grid_constant__ CUtensorMap tAh2, const __grid_constant__ CUtensorMap tAl2,
                       const __grid_constant__ CUtensorMap tBh2, const __grid_constant__ CUtensorMap tBl2, int M,
                       int N, int K, int K0, float alpha, float beta, float* C, int64_t ldc, int lower, int nprod,
                       int64_t ntiles, int* err, const EpiArgs ep, const __grid_constant__ GroupParam<G> gp) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES];
    __shared__ __align__(8) uint64_t tfull_bar[2], tempty_bar[2], fin_bar;
    __shared__ uint32_t tmem_holder;
    __shared__ volatile int s_abort;
    __shared__ int64_t s_issued, s_consumed;
    const uint32_t sbase = (dev::smem_u32(smem_raw) + 1023u) & ~1023u;   // 1024-byte aligned ring
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int tiles_m = (M + BM - 1) / BM;
    const int nk0 = (K0 + BK - 1) / BK;                       // chunks of the first segment
    const int nk = nk0 + (K - K0 + BK - 1) / BK;
    // Programmatic dependent launch: the next kernel in the stream may be scheduled now (it waits for this
    // grid's completion before touching memory); no-op when not launched with that attribute.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (threadIdx.x == 0) {
        // descriptor fetches overlap the setup below
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tAh)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tBh)) : "memory");
        if (nprod == 3) {
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tAl)) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tBl)) : "memory");
        }
        for (int s = 0; s < STAGES; ++s) {
            dev::mbar_init(&full_bar[s], 1);
            dev::mbar_init(&empty_bar[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            dev::mbar_init(&tfull_bar[a], 1);
            dev::mbar_init(&tempty_bar[a], EPI_WARPS);
        }
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
    // the previous kernel's writes (operands, C) are complete and visible past this point
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t tmem = tmem_holder;
    const uint32_t bytes_per_stage = (nprod == 3 ? 4u : 2u) * TILE_BYTES;

    if (warp == 0) {
        if (lane == 0) {   // ---- TMA producer
            int64_t g = 0;
            for (int64_t t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x) {
                const TileJob tj = tile_job<G>(t, gp, tiles_m, lower, M, N, nk, C, ldc, ep.Cr);
                const int tm = tj.tm, tn = tj.tn;
                for (int c = 0; c < tj.nk; ++c, ++g) {
                    const int slot = (int)(g % STAGES);
                    if (!wait_or_abort(&empty_bar[slot], (uint32_t)(((g / STAGES) & 1) ^ 1), &s_abort)) {
                        s_abort = 1;
                        break;
                    }
                    const uint32_t st = sbase + slot * STAGE_BYTES;
                    dev::mbar_expect_tx(&full_bar[slot], bytes_per_stage);
                    if constexpr (G) {
                        const GroupEntry& e = gp.g[tj.p];
                        const bool s2 = e.set != 0;
                        const int xa = e.ax + c * BK, xb = e.bx + c * BK;
                        tma_load_2d(st, s2 ? &tAh2 : &tAh, xa, e.ay_h + tm * BM, &full_bar[slot]);
                        tma_load_2d(st + 2 * TILE_BYTES, s2 ? &tBh2 : &tBh, xb, e.by_h + tn * BN, &full_bar[slot]);
                        tma_load_2d(st + TILE_BYTES, s2 ? &tAl2 : &tAl, xa, e.ay_l + tm * BM, &full_bar[slot]);
                        tma_load_2d(st + 3 * TILE_BYTES, s2 ? &tBl2 : &tBl, xb, e.by_l + tn * BN, &full_bar[slot]);
                    } else {
                        const bool seg2 = c >= nk0;
                        const int x = (seg2 ? c - nk0 : c) * BK;
                        tma_load_2d(st, seg2 ? &tAh2 : &tAh, x, tm * BM, &full_bar[slot]);
                        tma_load_2d(st + 2 * TILE_BYTES, seg2 ? &tBh2 : &tBh, x, tn * BN, &full_bar[slot]);
                        if (nprod == 3) {
                            tma_load_2d(st + TILE_BYTES, seg2 ? &tAl2 : &tAl, x, tm * BM, &full_bar[slot]);
                            tma_load_2d(st + 3 * TILE_BYTES, seg2 ? &tBl2 : &tBl, x, tn * BN, &full_bar[slot]);
                        }
                    }
                    s_issued = g + 1;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // ---- MMA issuer
            int64_t g = 0, lt = 0;
            bool ok = true;
            for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
                const uint32_t ab = (uint32_t)(lt & 1), aph = (uint32_t)((lt >> 1) & 1);
                if (!wait_or_abort(&tempty_bar[ab], aph ^ 1u, &s_abort)) {
                    ok = false;
                    break;
                }
                fence_after();
                const uint32_t acc = tmem + ab * BN;
                const int tnk = G ? tile_job<G>(t, gp, tiles_m, lower, M, N, nk, C, ldc, ep.Cr).nk : nk;
                for (int c = 0; c < tnk; ++c, ++g) {
                    const int slot = (int)(g % STAGES);
                    if (!wait_or_abort(&full_bar[slot], (uint32_t)((g / STAGES) & 1), &s_abort)) {
                        ok = false;
                        break;
                    }
                    s_consumed = g + 1;
                    fence_after();
                    const uint32_t st = sbase + slot * STAGE_BYTES;
                    const uint64_t dAh = sdesc_sw128(st), dAl = sdesc_sw128(st + TILE_BYTES);
                    const uint64_t dBh = sdesc_sw128(st + 2 * TILE_BYTES), dBl = sdesc_sw128(st + 3 * TILE_BYTES);
#pragma unroll
                    for (int kk = 0; kk < BK / 8; ++kk) {
                        const uint64_t off = (uint64_t)(kk * 32) >> 4;   // 8 TF32 = 32 bytes along the swizzled row
                        mma_tf32(acc, dAh + off, dBh + off, (c | kk) != 0 ? 1u : 0u);
                        if (nprod == 3) {
                            mma_tf32(acc, dAh + off, dBl + off, 1u);
                            mma_tf32(acc, dAl + off, dBh + off, 1u);
                        }
                    }
                    mma_commit(&empty_bar[slot]);   // the stage is free once these products are done
                }
                if (!ok) break;
                mma_commit(&tfull_bar[ab]);         // the accumulator is complete
            }
            if (!ok) s_abort = 1;
            mma_commit(&fin_bar);                   // arrives once every product issued above has completed
            if (!dev::mbar_wait_bounded(&fin_bar, 0)) s_abort = 1;
        }
    } else {   // ---- epilogue: warp w owns TMEM lanes 32 * (w % 4) .. +31 and 64 of the 128 columns
        const int q = warp & 3;
        const int half = (warp - 2) / 4;
        int64_t lt = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
            const TileJob tj = tile_job<G>(t, gp, tiles_m, lower, M, N, nk, C, ldc, ep.Cr);
            const int tm = tj.tm, tn = tj.tn, Mt = tj.M;
            const uint32_t ab = (uint32_t)(lt & 1), aph = (uint32_t)((lt >> 1) & 1);
            const int row = tm * BM + q * 32 + lane;
            const int n0 = tn * BN + half * 64;
            // columns n0 + j, j < jmax, are written by this thread (inside C, lower triangle when asked)
            int jmax = row < Mt ? min(64, tj.N - n0) : 0;
            if (lower) jmax = min(jmax, row - n0 + 1);
            const int ld32 = tj.ldc;   // 64 * ldc fits in 32 bits (host-checked)
            float* const cp = tj.C + ((int64_t)row + (int64_t)n0 * ld32);
            // C of this tile into registers while its products run (independent loads, all in flight)
            float cv[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) cv[j] = (j < jmax && beta != 0.f) ? __ldcg(cp + j * ld32) : 0.f;
            bool ok = wait_or_abort(&tfull_bar[ab], aph, &s_abort);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld is warp-collective
            if (!ok) {
                if (lane == 0) s_abort = 1;
                break;
            }
            fence_after();
            // optional K-major TF32 head / remainder copy of rows >= s_row0 (row stride s_kpad, zero past N)
            float* const sh =
                (ep.Sh && row >= ep.s_row0 && row < M) ? ep.Sh + (int64_t)(row - ep.s_row0) * ep.s_kpad + n0 : nullptr;
            float* const crp = tj.Cr ? tj.Cr + (cp - tj.C) : nullptr;
            // optional transposed copy of the band [x_row0, x_row0 + 128): column j -> row j
            const bool xband = ep.Xh && row >= ep.x_row0 && row < ep.x_row0 + BM;
            const int xmax = xband ? min(64, N - n0) : 0;
            float* const xh = xband ? ep.Xh + ((int64_t)n0 * BM + (row - ep.x_row0)) : nullptr;
            float* const xl = xband ? ep.Xl + (xh - ep.Xh) : nullptr;
            // 16 columns per step in a loop that is not unrolled: the tile's instructions are fetched once
            // (a fully unrolled 64-column epilogue spent most of a tile's time on instruction fetch); the
            // prefetched C values move down by 16 registers per step, so cv[0..15] are the step's columns
            const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + ab * BN + (uint32_t)(half * 64);
#pragma unroll 1
            for (int jb = 0; jb < 64; jb += 16) {
                uint32_t r[16];
                tmem_ld16(tb + (uint32_t)jb, r);
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = fmaf(alpha, __uint_as_float(r[j]), beta * cv[j]);
                float* const cpj = cp + jb * ld32;
                if (crp) {
                    float* const crj = crp + jb * ld32;
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (jb + j < jmax) {
                            const float h = __uint_as_float(__float_as_uint(v[j]) & 0xFFFFE000u);
                            __stcg(cpj + j * ld32, h);
                            __stcg(crj + j * ld32, v[j] - h);
                        }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (jb + j < jmax) __stcg(cpj + j * ld32, v[j]);
                }
                if (jb < xmax) {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (jb + j < xmax) {
                            const float x = row < Mt ? v[j] : 0.f;
                            const float h = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
                            xh[(int64_t)(jb + j) * BM] = h;
                            xl[(int64_t)(jb + j) * BM] = x - h;
                        }
                }
                if (sh && n0 + jb < ep.s_kpad) {
                    float* const shc = sh + jb;
                    float* const slc = ep.Sl + (shc - ep.Sh);
#pragma unroll
                    for (int j4 = 0; j4 < 4; ++j4) {
                        float h[4], l[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const float x = (jb + 4 * j4 + u < jmax) ? v[4 * j4 + u] : 0.f;
                            h[u] = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
                            l[u] = x - h[u];
                        }
                        reinterpret_cast<float4*>(shc)[j4] = make_float4(h[0], h[1], h[2], h[3]);
                        reinterpret_cast<float4*>(slc)[j4] = make_float4(l[0], l[1], l[2], l[3]);
                    }
                }
#pragma unroll
                for (int j = 0; j < 48; ++j) cv[j] = cv[j + 16];
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty_bar[ab]);   // accumulator free for the tile after next
        }
    }
    __syncthreads();
    if (s_abort) {
        if (threadIdx.x == 0) {
            atomicExch(err, -8 /* OMG_ERR_TIMEOUT */);
            for (int64_t g = s_consumed; g < s_issued; ++g)   // let copies in flight land before the CTA exits
                dev::mbar_wait_bounded(&full_bar[g % STAGES], (uint32_t)((g / STAGES) & 1));
        }
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// K-major FP32 matrix: `rows` rows of `k_extent` elements, row stride `ld` elements.
static CUtensorMap make_map(const float* base, int64_t rows, int64_t k_extent, int64_t ld) {
    return make_map_2d(base, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, rows, k_extent, ld, BK, BM);
}

}  // namespace tc

static inline void check_tc(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}

// Launch of the kernel; with `pdl` (programmatic dependent launch) it may be
// scheduled while the previous kernel in the stream finishes: the kernel
// waits for that kernel's completion before it touches memory.
template <bool G = false, typename... Args>
static void launch_gemm(bool pdl, unsigned grid, cudaStream_t s, Args... args) {
    if (!pdl) {
        tc::gemm_tf32x3_kernel<G><<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(tc::THREADS);
    cfg.dynamicSmemBytes = tc::SMEM_BYTES;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, tc::gemm_tf32x3_kernel<G>, args...);
}

// Checks the optional epilogue outputs against the shape and packs them.
static tc::EpiArgs epi_args(int64_t M, float beta, bool lower, int64_t N, float* Sh, float* Sl, int64_t s_row0,
                            int s_kpad, float* Cr, float* Xh, float* Xl, int64_t x_row0) {
    if (Sh) {   // the copy covers whole 128-column tiles: one tile column, 16-byte aligned rows
        if (!Sl || lower || N > tc::BN || s_kpad != tc::BN || s_row0 < 0 ||
            (reinterpret_cast<uintptr_t>(Sh) % 16) || (reinterpret_cast<uintptr_t>(Sl) % 16))
            throw Error(OMG_ERR_INVALID, "tensor-core GEMM split copy: unsupported shape");
    }
    if (Cr && beta != 0.f) throw Error(OMG_ERR_INVALID, "tensor-core GEMM head/remainder output needs beta = 0");
    if (Xh && (!Xl || lower || x_row0 < 0 || x_row0 % tc::BM || (M > 0 && x_row0 >= M)))
        throw Error(OMG_ERR_INVALID, "tensor-core GEMM band copy: unsupported shape");
    return tc::EpiArgs{Sh, Sl, Cr, Xh, Xl, (int)s_row0, s_kpad, (int)x_row0};
}

// C(M x N, ldc) = beta*C + alpha * A B^T.  A: M x K (K-major, row stride lda),
// B: N x K (K-major, row stride ldb); *h are TF32 heads, *l the remainders
// (may be null when nprod == 1).  `k0` offsets the K coordinate of A and B.
void gemm_tf32x3(int64_t M, int64_t N, int64_t K, float alpha, const float* Ah, const float* Al, int64_t lda,
                 int64_t a_kext, int64_t a_k0, const float* Bh, const float* Bl, int64_t ldb, int64_t b_kext,
                 int64_t b_k0, float beta, float* C, int64_t ldc, bool lower, int* err, cudaStream_t s,
                 const char* prof_name, int max_ctas, float* Sh, float* Sl, int64_t s_row0, int s_kpad, float* Cr,
                 float* Xh, float* Xl, int64_t x_row0, bool pdl) {
    const tc::EpiArgs ep = epi_args(M, beta, lower, N, Sh, Sl, s_row0, s_kpad, Cr, Xh, Xl, x_row0);
    if (M <= 0 || N <= 0) return;
    if (K <= 0) throw Error(OMG_ERR_INVALID, "empty K");
    ProfScope prof_(prof_name, s);
    const int nprod = (Al && Bl) ? 3 : 1;
    // Operands are offset along K by moving the base pointer (k0 multiple of 4 keeps 16-byte alignment).
    if ((a_k0 % 4) || (b_k0 % 4)) throw Error(OMG_ERR_INVALID, "tensor-core K offset not 16-byte aligned");
    const CUtensorMap mAh = tc::make_map(Ah + a_k0, M, a_kext - a_k0, lda);
    const CUtensorMap mAl = nprod == 3 ? tc::make_map(Al + a_k0, M, a_kext - a_k0, lda) : mAh;
    const CUtensorMap mBh = tc::make_map(Bh + b_k0, N, b_kext - b_k0, ldb);
    const CUtensorMap mBl = nprod == 3 ? tc::make_map(Bl + b_k0, N, b_kext - b_k0, ldb) : mBh;
    static bool attr = false;
    static int n_sm = 0;
    if (!attr) {
        cudaFuncSetAttribute(tc::gemm_tf32x3_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             tc::SMEM_BYTES);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (n_sm <= 0) n_sm = 1;
        attr = true;
    }
    if (lower && M != N) throw Error(OMG_ERR_INVALID, "lower-triangle tensor-core update needs M == N");
    if (ldc > (int64_t)(1 << 24)) throw Error(OMG_ERR_UNSUPPORTED, "tensor-core GEMM leading dimension too large");
    const int64_t tiles_m = (M + tc::BM - 1) / tc::BM, tiles_n = (N + tc::BN - 1) / tc::BN;
    if (tiles_m > (1 << 30) / 2) throw Error(OMG_ERR_UNSUPPORTED, "tensor-core GEMM too tall");
    const int64_t ntiles = lower ? tiles_m * (tiles_m + 1) / 2 : tiles_m * tiles_n;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, max_ctas > 0 ? std::min(max_ctas, n_sm) : n_sm);
    launch_gemm(pdl, grid, s, mAh, mAl, mBh, mBl, mAh, mAl, mBh, mBl, (int)M, (int)N, (int)K, (int)K, alpha, beta, C,
                ldc, lower ? 1 : 0, nprod, ntiles, err, ep, tc::GroupParam<false>{0});
    check_tc("gemm_tf32x3");
}

// C(M x N, ldc) = beta C + alpha (A1 B1^T + A2 B2^T): two K segments (K1, K2, each
// a multiple of 32 but the last) in one pass over C; all operands split
// (3xTF32), K-major with row strides lda1 / ldb1 / lda2 / ldb2.
void gemm_tf32x3_pair(int64_t M, int64_t N, float alpha, int64_t K1, const float* A1h, const float* A1l, int64_t lda1,
                      const float* B1h, const float* B1l, int64_t ldb1, int64_t K2, const float* A2h,
                      const float* A2l, int64_t lda2, const float* B2h, const float* B2l, int64_t ldb2, float beta,
                      float* C, int64_t ldc, bool lower, int* err, cudaStream_t s, const char* prof_name,
                      int max_ctas, float* Sh, float* Sl, int64_t s_row0, int s_kpad, bool pdl) {
    const tc::EpiArgs ep = epi_args(M, beta, lower, N, Sh, Sl, s_row0, s_kpad, nullptr, nullptr, nullptr, 0);
    if (M <= 0 || N <= 0) return;
    if (K1 <= 0 || K2 <= 0 || (K1 % tc::BK)) throw Error(OMG_ERR_INVALID, "tensor-core GEMM segments");
    ProfScope prof_(prof_name, s);
    const CUtensorMap m1h = tc::make_map(A1h, M, K1, lda1), m1l = tc::make_map(A1l, M, K1, lda1);
    const CUtensorMap n1h = tc::make_map(B1h, N, K1, ldb1), n1l = tc::make_map(B1l, N, K1, ldb1);
    const CUtensorMap m2h = tc::make_map(A2h, M, K2, lda2), m2l = tc::make_map(A2l, M, K2, lda2);
    const CUtensorMap n2h = tc::make_map(B2h, N, K2, ldb2), n2l = tc::make_map(B2l, N, K2, ldb2);
    static bool attr = false;
    static int n_sm = 0;
    if (!attr) {
        cudaFuncSetAttribute(tc::gemm_tf32x3_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             tc::SMEM_BYTES);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (n_sm <= 0) n_sm = 1;
        attr = true;
    }
    if (lower && M != N) throw Error(OMG_ERR_INVALID, "lower-triangle tensor-core update needs M == N");
    if (ldc > (int64_t)(1 << 24)) throw Error(OMG_ERR_UNSUPPORTED, "tensor-core GEMM leading dimension too large");
    const int64_t tiles_m = (M + tc::BM - 1) / tc::BM, tiles_n = (N + tc::BN - 1) / tc::BN;
    const int64_t ntiles = lower ? tiles_m * (tiles_m + 1) / 2 : tiles_m * tiles_n;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, max_ctas > 0 ? std::min(max_ctas, n_sm) : n_sm);
    launch_gemm(pdl, grid, s, m1h, m1l, n1h, n1l, m2h, m2l, n2h, n2l, (int)M, (int)N, (int)(K1 + K2), (int)K1, alpha,
                beta, C, ldc, lower ? 1 : 0, 3, ntiles, err, ep, tc::GroupParam<false>{0});
    check_tc("gemm_tf32x3");
}

// Independent products C_p = alpha A_p B_p^T (3xTF32, heads into C_p, remainders into Cr_p), all read through
// two sets of four operand maps (Ah, Al, Bh, Bl: K-major FP32, `rows` rows of `kext` elements, row stride
// `ld`) at the products' own coordinates; one persistent launch per MAX_GROUP products instead of one launch
// per product.  Each product's tiles read only operand rows and write only outputs of their own (the caller
// guarantees that products do not overlap in what they write nor write what another reads).
void gemm_tf32x3_grouped(const GemmOperand ops[8], const std::vector<GemmProduct>& prods, float alpha, int* err,
                         cudaStream_t s, const char* prof_name, bool pdl) {
    if (prods.empty()) return;
    ProfScope prof_(prof_name, s);
    CUtensorMap maps[8];
    for (int i = 0; i < 8; ++i) {
        if (!ops[i].base || ops[i].rows <= 0 || ops[i].kext <= 0)
            throw Error(OMG_ERR_INVALID, "grouped tensor-core GEMM: empty operand map");
        if (ops[i].rows > INT32_MAX || ops[i].kext > INT32_MAX)
            throw Error(OMG_ERR_UNSUPPORTED, "grouped tensor-core GEMM: operand too large for 32-bit coordinates");
        maps[i] = tc::make_map(ops[i].base, ops[i].rows, ops[i].kext, ops[i].ld);
    }
    static bool attr = false;
    static int n_sm = 0;
    if (!attr) {
        cudaFuncSetAttribute(tc::gemm_tf32x3_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             tc::SMEM_BYTES);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (n_sm <= 0) n_sm = 1;
        attr = true;
    }
    auto gp = std::make_unique<tc::GroupParam<true>>();
    for (size_t b0 = 0; b0 < prods.size(); b0 += tc::MAX_GROUP) {
        const size_t b1 = std::min(prods.size(), b0 + (size_t)tc::MAX_GROUP);
        int64_t ntiles = 0;
        gp->n = 0;
        for (size_t i = b0; i < b1; ++i) {
            const GemmProduct& q = prods[i];
            if (q.M <= 0 || q.N <= 0) continue;
            if (q.K <= 0 || q.set < 0 || q.set > 1 || !q.C || !q.Cr || q.ldc <= 0 || q.ldc > (int64_t)(1 << 24) ||
                q.ax % 4 || q.bx % 4 || q.ax < 0 || q.bx < 0 || q.ay_h < 0 || q.ay_l < 0 || q.by_h < 0 || q.by_l < 0)
                throw Error(OMG_ERR_INVALID, "grouped tensor-core GEMM: bad product");
            const int64_t t = ((q.M + tc::BM - 1) / tc::BM) * ((q.N + tc::BN - 1) / tc::BN);
            if (ntiles + t > INT32_MAX) throw Error(OMG_ERR_UNSUPPORTED, "grouped tensor-core GEMM: too many tiles");
            tc::GroupEntry& e = gp->g[gp->n++];
            e = tc::GroupEntry{q.C,       q.Cr,      (int)q.ldc, (int)q.M,  (int)q.N,  (int)q.K,  q.set,
                               (int)q.ay_h, (int)q.ay_l, (int)q.by_h, (int)q.by_l, (int)q.ax, (int)q.bx, (int)ntiles};
            ntiles += t;
        }
        if (gp->n == 0) continue;
        const unsigned grid = (unsigned)std::min<int64_t>(ntiles, n_sm);
        const tc::EpiArgs ep{nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0, 0};
        launch_gemm<true>(pdl, grid, s, maps[0], maps[1], maps[2], maps[3], maps[4], maps[5], maps[6], maps[7], 0, 0,
                          0, 0, alpha, 0.f, (float*)nullptr, (int64_t)0, 0, 3, ntiles, err, ep, *gp);
        check_tc("gemm_tf32x3_grouped");
    }
}

// ---------------------------------------------------------------------------
// Operand splitting: X = Xh + Xl with Xh = X with its low 13 mantissa bits
// cleared (exactly representable in TF32) and Xl = X - Xh (exact in FP32).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void split_tf32(float x, float& h, float& l) {
    h = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    l = x - h;
}

// Column-major panel P (m x nk, ld) -> K-major (row-major) heads/remainders
// (m x kpad, row stride kpad), zero beyond nk.  32 x 32 tiles through shared
// memory so both reads and writes are coalesced.
__global__ void split_panel_kmajor_kernel(int64_t m, int nk, int kpad, const float* __restrict__ P, int64_t ld,
                                          float* H, float* L) {
    __shared__ float t[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int k0 = blockIdx.y * 32;
    for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
        const int64_t i = i0 + threadIdx.x;
        const int k = k0 + kk;
        t[kk][threadIdx.x] = (i < m && k < nk) ? P[i + (int64_t)k * ld] : 0.f;
    }
    __syncthreads();
    for (int ii = threadIdx.y; ii < 32; ii += blockDim.y) {
        const int64_t i = i0 + ii;
        const int k = k0 + threadIdx.x;
        if (i < m && k < kpad) {
            float h, l;
            split_tf32(t[threadIdx.x][ii], h, l);
            H[i * kpad + k] = h;
            L[i * kpad + k] = l;
        }
    }
}

void split_panel_kmajor(int64_t m, int nk, int kpad, const float* P, int64_t ld, float* H, float* L,
                        cudaStream_t s) {
    if (m <= 0) return;
    ProfScope prof_("split_panel", s);
    dim3 grid((unsigned)((m + 31) / 32), (unsigned)((kpad + 31) / 32));
    split_panel_kmajor_kernel<<<grid, dim3(32, 8), 0, s>>>(m, nk, kpad, P, ld, H, L);
    check_tc("split_panel");
}

// Column-major block X (nk x ncol, ldx): column j becomes K-major row j of
// (ncol x kpad) heads/remainders.
__global__ void split_cols_kernel(int nk, int64_t ncol, int kpad, const float* __restrict__ X, int64_t ldx, float* H,
                                  float* L) {
    for (int64_t j = blockIdx.y; j < ncol; j += gridDim.y) {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kpad; k += gridDim.x * blockDim.x) {
            const float v = k < nk ? X[k + j * ldx] : 0.f;
            float h, l;
            split_tf32(v, h, l);
            H[j * kpad + k] = h;
            L[j * kpad + k] = l;
        }
    }
}

void split_cols(int nk, int64_t ncol, int kpad, const float* X, int64_t ldx, float* H, float* L, cudaStream_t s) {
    if (ncol <= 0) return;
    ProfScope prof_("split_cols", s);
    dim3 grid((unsigned)((kpad + 127) / 128), (unsigned)std::min<int64_t>(ncol, 65535));
    split_cols_kernel<<<grid, 128, 0, s>>>(nk, ncol, kpad, X, ldx, H, L);
    check_tc("split_cols");
}

}  // namespace omg

// Test hook (not part of the public header): the tensor-core GEMM on caller
// operands, for the unit tests of the kernel itself.
extern "C" int omg_internal_gemm_tf32x3(int64_t M, int64_t N, int64_t K, float alpha, const float* Ah,
                                        const float* Al, int64_t lda, const float* Bh, const float* Bl, int64_t ldb,
                                        float beta, float* C, int64_t ldc, int lower, int* err) {
    try {
        omg::gemm_tf32x3(M, N, K, alpha, Ah, Al, lda, K, 0, Bh, Bl, ldb, K, 0, beta, C, ldc, lower != 0, err, 0,
                         "gemm_tf32x3", 0, nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr, 0, false);
        cudaError_t e = cudaDeviceSynchronize();
        return e == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        return e.code;
    }
}

// Test hook: the same with the K-major TF32 split copy of C's rows >= s_row0
// written by the epilogue (N <= 128, row stride 128).
extern "C" int omg_internal_gemm_tf32x3_split(int64_t M, int64_t N, int64_t K, float alpha, const float* Ah,
                                              const float* Al, int64_t lda, const float* Bh, const float* Bl,
                                              int64_t ldb, float beta, float* C, int64_t ldc, float* Sh, float* Sl,
                                              int64_t s_row0, int* err) {
    try {
        omg::gemm_tf32x3(M, N, K, alpha, Ah, Al, lda, K, 0, Bh, Bl, ldb, K, 0, beta, C, ldc, false, err, 0,
                         "gemm_tf32x3", 0, Sh, Sl, s_row0, 128, nullptr, nullptr, nullptr, 0, false);
        cudaError_t e = cudaDeviceSynchronize();
        return e == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        return e.code;
    }
}

// Test hook: the same with C written as TF32 heads and Cr as the remainders
// (when Cr is not null, beta = 0) and/or the transposed head / remainder copy
// of the 128-row band of C at x_row0 (Xh/Xl: N rows of 128, zero past M).
extern "C" int omg_internal_gemm_tf32x3_epi(int64_t M, int64_t N, int64_t K, float alpha, const float* Ah,
                                            const float* Al, int64_t lda, const float* Bh, const float* Bl,
                                            int64_t ldb, float beta, float* C, int64_t ldc, float* Cr, float* Xh,
                                            float* Xl, int64_t x_row0, int* err) {
    try {
        omg::gemm_tf32x3(M, N, K, alpha, Ah, Al, lda, K, 0, Bh, Bl, ldb, K, 0, beta, C, ldc, false, err, 0,
                         "gemm_tf32x3", 0, nullptr, nullptr, 0, 0, Cr, Xh, Xl, x_row0, false);
        cudaError_t e = cudaDeviceSynchronize();
        return e == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        return e.code;
    }
}
