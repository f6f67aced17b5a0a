// Refinement residual R = B - A X with FP64-level accuracy on the bf16 tensor
// cores (sm_103a, tcgen05), by exact fixed-point slicing (the scheme of
// Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 59 (2012), in its
// fixed-point form):
//
//   A_ij = 2^(e_i) sum_s 2^(-beta s) alpha_s,ij     (row scale e_i, integer digits |alpha| <= 2^beta)
//   X_jc = 2^(f_c) sum_t 2^(-beta t) xi_t,jc        (column scale f_c)
//   (A X)_ic = 2^(e_i + f_c) sum_{s,t} 2^(-beta (s+t)) (alpha_s xi_t)_ic
//
// Every digit is an integer of at most beta+1 bits, exact in bf16; each
// product alpha_s xi_t is an integer GEMM.  The MMA accumulates in FP32, which
// is exact while partial sums stay below 2^24: the K dimension is cut into
// windows of KC = 256 (|partial sum| <= 256 * 2^(2 beta) = 2^22 for beta = 7),
// each window is read out of TMEM, converted to int32 (exact) and summed in
// registers; the digits of one level s+t are summed while the int32 bound
// allows, then the level is scaled and subtracted from R in FP64.  Digit
// pairs are kept up to level s+t <= LMAX; with beta = 7, 7 digits per operand
// and LMAX = 8, truncated digits and dropped levels stay near 2^-48 of
// n max|A_i.| max|X_.c| per entry, far under the refinement's needs (the head
// matrix itself carries the mixed assembly's ~1e-8 error).
//
// Persistent and warp-specialized like the 3xTF32 GEMM: warp 0 streams
// 128 x 64 bf16 tiles of the A digits and up to 256 x 64 tiles of the X
// digits (TMA, 128-byte swizzle) through a three-stage ring, warp 1 issues
// tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = nmma <= 256, K = 16) into
// two TMEM accumulators of 256 columns (one per window, alternating), warps
// 2-17 drain the windows (warp w: TMEM lanes 32 (w % 4) .. +31, columns
// 64 ((w - 2) / 4) .. +63).  An output tile covers up to 256 columns, so a
// residual with <= 256 right-hand sides streams each A digit plane once per
// digit pair it takes part in (3.5 times per plane on average for 21 pairs
// of 6 digits), not once per pair and 128-column block.  Keeping the level
// sums of all six levels on chip at once, which would stream each plane once,
// needs 6 accumulators of the tile's width: more than the 512 TMEM columns.
// Output tiles of one row block are adjacent in the walk, so the CTAs that
// share a row block stream the same A digits at the same time (L2 reuse).
// Every wait is bounded; on timeout the kernel records OMG_ERR_TIMEOUT, all
// roles stop, copies and products in flight are waited for, TMEM is released.
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "handles.h"
#include "tcgen05.cuh"

namespace omg {
namespace tcr {

using tc::fence_after;
using tc::fence_before;

constexpr int BM = 128, BN = 256, BK = 64;        // BN: widest tile (MMA N); BK bf16 = 128 bytes per swizzled row
constexpr int STAGES = 3;
constexpr int TILE_A = BM * BK * 2;               // 16 KiB
constexpr int TILE_X = BN * BK * 2;               // 32 KiB (room for the widest tile)
constexpr int STAGE_BYTES = TILE_A + TILE_X;
constexpr int EPI_WARPS = 16;
constexpr int THREADS = 64 + EPI_WARPS * 32;      // 576
constexpr int SPILL = 32;                         // level-sum columns a thread hands to the FP64 pass at a time
constexpr int SMEM_INT_BYTES = SPILL * EPI_WARPS * 32 * 4;   // 64 KiB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + SMEM_INT_BYTES + 1024;
constexpr uint32_t TMEM_COLS = 512;
constexpr int KC = 256;                           // exact-accumulation window
constexpr int CPW = KC / BK;                      // chunks per window
constexpr int MAXPAIRS = 64;
constexpr int MAXRANGES = 8;

// Rows [beg[q], beg[q] + len[q]) concatenated (n == 0: all rows in order).
struct RowRanges {
    int n;
    int64_t beg[MAXRANGES], len[MAXRANGES];
};

// Instruction descriptor: D=F32, A=B=BF16, both K-major, M=128, N=n (a multiple of 16, <= 256).
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

constexpr int MAXGROUPS = 6;

struct PairPlan {
    int n;                       // digit pairs, ordered by level s + t
    int ngroups;                 // work items per output tile: level-aligned runs of pairs, each summed into its
    int gbeg[MAXGROUPS + 1];     // own output slice (pairs gbeg[g] .. gbeg[g + 1] - 1)
    int nwin;                    // windows per pair (K = nwin * KC, zero-padded)
    uint64_t flush;              // bit p: subtract the level sum after pair p
    uint8_t s[MAXPAIRS], t[MAXPAIRS];
};

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__global__ void __launch_bounds__(THREADS, 1)
    residual_slices_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tX,
                           const __grid_constant__ PairPlan plan, int N, int k, int kpad, int beta,
                           const int* __restrict__ rexp, const int* __restrict__ cexp, double sgn, double* R,
                           int64_t ldr, double* Rp, int64_t ntiles, int nrb, int ncb, int nmma, int* err) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES];
    __shared__ __align__(8) uint64_t tfull_bar[2], tempty_bar[2], fin_bar;
    __shared__ uint32_t tmem_holder;
    __shared__ volatile int s_abort;
    __shared__ int64_t s_issued, s_consumed;
    const uint32_t sbase = (dev::smem_u32(smem_raw) + 1023u) & ~1023u;
    int* const s_int = reinterpret_cast<int*>(smem_raw + (sbase - dev::smem_u32(smem_raw)) + STAGES * STAGE_BYTES);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (threadIdx.x == 0) {
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
    const uint32_t tmem = tmem_holder;

    if (warp == 0) {
        if (lane == 0) {   // ---- TMA producer
            int64_t g = 0;
            for (int64_t t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x) {
                const int gr = (int)(t / ((int64_t)nrb * ncb)), rb = (int)(t / ncb % nrb), cb = (int)(t % ncb);
                const int units = (plan.gbeg[gr + 1] - plan.gbeg[gr]) * plan.nwin;
                for (int u = 0; u < units && !s_abort; ++u) {
                    const int p = plan.gbeg[gr] + u / plan.nwin, w = u % plan.nwin;
                    const int ya = (plan.s[p] - 1) * N + rb * BM, yx = (plan.t[p] - 1) * kpad + cb * nmma;
                    for (int c = 0; c < CPW; ++c, ++g) {
                        const int slot = (int)(g % STAGES);
                        if (!tc::wait_or_abort(&empty_bar[slot], (uint32_t)(((g / STAGES) & 1) ^ 1), &s_abort)) {
                            s_abort = 1;
                            break;
                        }
                        const uint32_t st = sbase + slot * STAGE_BYTES;
                        const int x = (w * CPW + c) * BK;
                        dev::mbar_expect_tx(&full_bar[slot], TILE_A + nmma * BK * 2);
                        tc::tma_load_2d(st, &tA, x, ya, &full_bar[slot]);
                        tc::tma_load_2d(st + TILE_A, &tX, x, yx, &full_bar[slot]);
                        s_issued = g + 1;
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // ---- MMA issuer
            int64_t g = 0, lu = 0;
            bool ok = true;
            const uint32_t idesc = idesc_bf16(nmma);
            for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int gr = (int)(t / ((int64_t)nrb * ncb));
                const int units = (plan.gbeg[gr + 1] - plan.gbeg[gr]) * plan.nwin;
                for (int u = 0; u < units && ok; ++u, ++lu) {
                    const uint32_t ab = (uint32_t)(lu & 1), aph = (uint32_t)((lu >> 1) & 1);
                    if (!tc::wait_or_abort(&tempty_bar[ab], aph ^ 1u, &s_abort)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t acc = tmem + ab * BN;
                    for (int c = 0; c < CPW; ++c, ++g) {
                        const int slot = (int)(g % STAGES);
                        if (!tc::wait_or_abort(&full_bar[slot], (uint32_t)((g / STAGES) & 1), &s_abort)) {
                            ok = false;
                            break;
                        }
                        s_consumed = g + 1;
                        fence_after();
                        const uint32_t st = sbase + slot * STAGE_BYTES;
                        const uint64_t dA = tc::sdesc_sw128(st), dX = tc::sdesc_sw128(st + TILE_A);
#pragma unroll
                        for (int kk = 0; kk < BK / 16; ++kk) {
                            const uint64_t off = (uint64_t)(kk * 32) >> 4;   // 16 bf16 = 32 bytes
                            mma_bf16(acc, dA + off, dX + off, idesc, (c | kk) != 0 ? 1u : 0u);
                        }
                        tc::mma_commit(&empty_bar[slot]);
                    }
                    if (!ok) break;
                    tc::mma_commit(&tfull_bar[ab]);   // the window's exact partial sums are ready
                }
            }
            if (!ok) s_abort = 1;
            tc::mma_commit(&fin_bar);
            if (!dev::mbar_wait_bounded(&fin_bar, 0)) s_abort = 1;
        }
    } else {   // ---- epilogue: warp w owns TMEM lanes 32 (w % 4) .. +31 and columns 64 ((w - 2) / 4) .. +63
        const int q = warp & 3;
        const int grp = (warp - 2) >> 2;
        const bool active = grp * 64 < nmma;   // warp-uniform: columns past the MMA width hold nothing
        int* const si = s_int + (warp - 2) * 32 + lane;
        int64_t lu = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int gr = (int)(t / ((int64_t)nrb * ncb)), rb = (int)(t / ncb % nrb), cb = (int)(t % ncb);
            const int units = (plan.gbeg[gr + 1] - plan.gbeg[gr]) * plan.nwin;
            const int row = rb * BM + q * 32 + lane;
            const int c0 = cb * nmma + grp * 64;
            const int cend = min(64, nmma - grp * 64);   // the group's columns inside this tile
            const int er = row < N ? rexp[row] : 0;
            int iacc[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) iacc[j] = 0;
            bool stop = false;
            for (int u = 0; u < units; ++u, ++lu) {
                const uint32_t ab = (uint32_t)(lu & 1), aph = (uint32_t)((lu >> 1) & 1);
                bool ok = tc::wait_or_abort(&tfull_bar[ab], aph, &s_abort);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) {
                    if (lane == 0) s_abort = 1;
                    stop = true;
                    break;
                }
                fence_after();
                if (active) {
#pragma unroll
                    for (int chunk = 0; chunk < 4; ++chunk) {
                        uint32_t r[16];
                        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + ab * BN + (uint32_t)(grp * 64 + chunk * 16),
                                      r);
#pragma unroll
                        for (int j = 0; j < 16; ++j)   // |window sum| < 2^22: adding 1.5 * 2^23 puts it in the mantissa
                            iacc[chunk * 16 + j] += __float_as_int(__uint_as_float(r[j]) + 12582912.0f) - 0x4B400000;
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&tempty_bar[ab]);
                const int p = plan.gbeg[gr] + u / plan.nwin, w = u % plan.nwin;
                if (active && w == plan.nwin - 1 && ((plan.flush >> p) & 1ull)) {   // level sum -> R (FP64)
                    // 32 columns at a time through shared memory, so the (rare) FP64 pass holds few registers
                    const int lev = plan.s[p] + plan.t[p];
                    // group 0 sums into R, group g > 0 into its own n x k slice of Rp (leading dimension N)
                    double* const Rg = gr == 0 ? R : Rp + (int64_t)(gr - 1) * N * k;
                    const int64_t ldg = gr == 0 ? ldr : N;
#pragma unroll
                    for (int h = 0; h < 64 / SPILL; ++h) {
#pragma unroll
                        for (int j = 0; j < SPILL; ++j) {
                            si[j * (EPI_WARPS * 32)] = iacc[h * SPILL + j];
                            iacc[h * SPILL + j] = 0;
                        }
                        if (row < N) {
                            for (int j = 0; j < SPILL; ++j) {
                                const int col = c0 + h * SPILL + j;
                                const int v = si[j * (EPI_WARPS * 32)];
                                if (h * SPILL + j < cend && col < k && v != 0) {
                                    Rg[row + (int64_t)col * ldg] +=
                                        sgn * scalbn((double)v, er + __ldg(cexp + col) - beta * lev);
                                }
                            }
                        }
                    }
                }
            }
            if (stop) break;
        }
    }
    __syncthreads();
    if (s_abort) {
        if (threadIdx.x == 0) {
            atomicExch(err, -8 /* OMG_ERR_TIMEOUT */);
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

// R += the ng partial sums of the level groups 1.. (n x k slices of P), in group order.
__global__ void sum_groups_kernel(int64_t n, int64_t k, int ng, const double* __restrict__ P, double* R, int64_t ldr) {
    for (int64_t j = blockIdx.y; j < k; j += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x) {
            double v = R[i + j * ldr];
            for (int g = 0; g < ng; ++g) v += P[g * n * k + i + j * n];
            R[i + j * ldr] = v;
        }
}

// Digits of the columns of a column-major FP64 matrix: column c (rows j < n)
// is scaled by 2^-e_c (e_c: exponent of its largest magnitude, frexp
// convention), rounded to a multiple of 2^-(nd beta) and cut into `nd`
// balanced base-2^beta digits (first |d| <= 2^beta, others <= 2^(beta-1)), written as bf16
// row c of digit plane d: out[(d * rows_per_plane + c) * ldo + j], zero for
// n <= j < ldo.  Columns c >= ncol (up to rows_per_plane) are zero.
// x 2^k rounded to the nearest integer (ties to even), exactly, by integer
// arithmetic on the bits of x (|x 2^k| < 2^62): the same value as
// __double2ll_rn(x * 2^k) without the FP64 pipe.
__device__ __forceinline__ long long scaled_rn(double x, int k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7FF);
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (E ? (1ull << 52) : 0ull);
    const int sh = (E ? E : 1) - 1075 + k;   // |x 2^k| = m 2^sh
    unsigned long long q;
    if (sh >= 0) {
        q = m << sh;
    } else if (sh < -63) {
        q = 0;   // below 2^-11
    } else {
        // t = m >> (r - 1) keeps the half bit as its lowest bit; the bits below it are the sticky part:
        // round up when the half bit is set and (anything below it is set, or q is odd)
        const int r1 = -sh - 1;
        const unsigned long long t = m >> r1;
        const unsigned long long sticky = (m & ((1ull << r1) - 1ull)) != 0ull ? 1ull : 0ull;
        q = t >> 1;
        q += t & (sticky | q) & 1ull;
    }
    return (b >> 63) ? -(long long)q : (long long)q;
}

// bf16 bits of a small integer (|r| < 2^8, exact in bf16): 1.5 * 2^23 + r
// has r in its low mantissa bits, the subtraction leaves float(r) exactly.
__device__ __forceinline__ unsigned short small_int_bf16(long long r) {
    const float f = __int_as_float(0x4B400000 + (int)r) - 12582912.0f;
    return (unsigned short)(__float_as_uint(f) >> 16);
}

// Digits of the columns of a column-major FP64 matrix: column c (rows j < n)
// is scaled by 2^-e_c (e_c: exponent of its largest magnitude, frexp
// convention), rounded to a multiple of 2^-(nd beta) and cut into `nd`
// balanced base-2^beta digits (first |d| <= 2^beta, others <= 2^(beta-1)), written as bf16
// row c of digit plane d: out[(d * rows_per_plane + c) * ldo + j], zero for
// n <= j < ldo.  Columns c >= ncol (up to rows_per_plane) are zero.  One CTA
// per column, four consecutive rows per thread (8-byte stores per plane);
// integer arithmetic only (the largest magnitude by its bit pattern, the
// scaling and rounding on the significand).  Optionally also writes the
// column's entries on and below the diagonal, rounded to FP32, to lower32.
constexpr int DG_THREADS = 256;

// ND_T / BETA_T > 0: the layout fixed at compile time (the digit shifts become immediates and the
// digit loop unrolls); 0: taken from nd / beta at run time.
template <int ND_T, int BETA_T>
__global__ void __launch_bounds__(DG_THREADS) digits_kernel(const double* __restrict__ M, int64_t n, int64_t ncol,
                                                            int64_t ldm, int nd_rt, int beta_rt, int64_t rows_per_plane,
                                                            int64_t ldo, __nv_bfloat16* out, int* ex,
                                                            const __grid_constant__ RowRanges rr, float* lower32,
                                                            int64_t ld32) {
    const int nd = ND_T > 0 ? ND_T : nd_rt, beta = BETA_T > 0 ? BETA_T : beta_rt;
    __shared__ unsigned long long red[DG_THREADS / 32];
    __shared__ int s_e;
    const int64_t c = blockIdx.x;
    uint2* const o2 = reinterpret_cast<uint2*>(out);   // 4 bf16 per store (ldo is a multiple of 64)
    if (c >= ncol) {
        for (int d = 0; d < nd; ++d)
            for (int64_t j = 4 * threadIdx.x; j < ldo; j += 4 * DG_THREADS)
                o2[(((int64_t)d * rows_per_plane + c) * ldo + j) / 4] = make_uint2(0u, 0u);
        return;
    }
    const double* col = M + c * ldm;
    // entry j of the digit row: row j of the column, or the j-th row of the ranges
    auto at = [&](int64_t j) -> double {
        if (rr.n == 0) return col[j];
        for (int q = 0; q < rr.n; ++q) {
            if (j < rr.len[q]) return col[rr.beg[q] + j];
            j -= rr.len[q];
        }
        return 0.0;
    };
    unsigned long long mb = 0;   // |x| bits: ordered like |x| for finite x
    for (int64_t j = threadIdx.x; j < n; j += DG_THREADS)
        mb = max(mb, (unsigned long long)__double_as_longlong(at(j)) & 0x7FFFFFFFFFFFFFFFull);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = mb;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = red[0];
        for (int w = 1; w < DG_THREADS / 32; ++w) m = max(m, red[w]);
        int e = 0;
        frexp(__longlong_as_double((long long)m), &e);   // max = f 2^e, f in [0.5, 1): every |entry| 2^-e < 1
        s_e = e;
        ex[c] = e;
    }
    __syncthreads();
    const int k = nd * beta - s_e;
    // one rounding to the digit grid 2^-(nd beta), then balanced base-2^beta digits by integer
    // arithmetic (|Y| <= 2^(nd beta) <= 2^62).  Taken one after the other, r = ((Y + h) & mask) - h,
    // Y <- (Y - r) >> beta (h = 2^(beta-1)); by induction the i-th remainder is
    // floor((Y + h sum_{j<i} 2^(beta j)) / 2^(beta i)), so with the bias Bs = h sum_{j<nd-1} 2^(beta j)
    // (extra terms only add multiples of 2^beta to the shifted value) the digits carry nothing:
    // digit i < nd-1 is ((Y + Bs) >> (beta i) & mask) - h and the top one (Y + Bs) >> (beta (nd-1)).
    const long long half = 1ll << (beta - 1);
    const unsigned mask = (1u << beta) - 1u;
    long long Bs = 0;
    for (int j = 0; j + 1 < nd; ++j) Bs += half << (beta * j);
    const int bf_off = 0x4B400000 - (int)half;   // float bits of 1.5 * 2^23 + (field - h)
    for (int64_t j0 = 4 * threadIdx.x; j0 < ldo; j0 += 4 * DG_THREADS) {
        long long Z[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double x = j0 + u < n ? at(j0 + u) : 0.0;
            Z[u] = (j0 + u < n ? scaled_rn(x, k) : 0) + Bs;
            if (lower32 && j0 + u >= c && j0 + u < n) lower32[j0 + u + c * ld32] = (float)x;   // lower triangle
        }
#pragma unroll
        for (int d = (ND_T > 0 ? ND_T : nd) - 1; d >= 0; --d) {
            const int sh = beta * (nd - 1 - d);
            unsigned int f[4];   // FP32 bits of the digits; their high halves are the bf16 values
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (d > 0) {   // float(1.5 * 2^23 + digit) - 1.5 * 2^23, exact
                    const unsigned field = (unsigned)(Z[u] >> sh) & mask;
                    f[u] = __float_as_uint(__int_as_float(bf_off + (int)field) - 12582912.0f);
                } else {
                    f[u] = (unsigned)small_int_bf16(Z[u] >> sh) << 16;
                }
            }
            o2[(((int64_t)d * rows_per_plane + c) * ldo + j0) / 4] =
                make_uint2(__byte_perm(f[0], f[1], 0x7632), __byte_perm(f[2], f[3], 0x7632));
        }
    }
}

}  // namespace tcr

static inline void check_tcr(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}

int64_t digits_ld(int64_t n) { return (n + 63) / 64 * 64; }

void digits_columns(const double* M, int64_t n, int64_t ncol, int64_t ldm, int nd, int beta, int64_t rows_per_plane,
                    int64_t ldo, void* out, int* ex, cudaStream_t s,
                    const std::vector<std::pair<int64_t, int64_t>>* ranges = nullptr, float* lower32 = nullptr,
                    int64_t ld32 = 0) {
    if (rows_per_plane <= 0) return;
    if (nd < 1 || nd * beta > 62 || beta < 2 || beta > 8 || ldo % 4 || ldo < n)
        throw Error(OMG_ERR_INVALID, "digits: bad digit layout");
    if (lower32 && (ranges || ld32 < n)) throw Error(OMG_ERR_INVALID, "digits: FP32 copy of a full square matrix only");
    ProfScope prof_("digits", s);
    tcr::RowRanges rr{};
    if (ranges) {
        if (ranges->size() > (size_t)tcr::MAXRANGES) throw Error(OMG_ERR_INVALID, "digits: too many row ranges");
        int64_t tot = 0;
        for (const auto& r : *ranges) {
            rr.beg[rr.n] = r.first;
            rr.len[rr.n] = r.second - r.first;
            tot += rr.len[rr.n++];
        }
        if (tot != n) throw Error(OMG_ERR_INVALID, "digits: row ranges do not add up");
    }
    if (nd == 6 && beta == 7)   // the library's layout
        tcr::digits_kernel<6, 7><<<(unsigned)rows_per_plane, tcr::DG_THREADS, 0, s>>>(
            M, n, ncol, ldm, nd, beta, rows_per_plane, ldo, static_cast<__nv_bfloat16*>(out), ex, rr, lower32, ld32);
    else
        tcr::digits_kernel<0, 0><<<(unsigned)rows_per_plane, tcr::DG_THREADS, 0, s>>>(
            M, n, ncol, ldm, nd, beta, rows_per_plane, ldo, static_cast<__nv_bfloat16*>(out), ex, rr, lower32, ld32);
    check_tcr("digits");
}

// R = B + sgn A X^T over a contraction of length kdim, both operands by their
// digit rows: A (n x kdim) as nda planes of n rows, X (k x kdim) as ndx planes
// of kpad rows, row stride ld = digits_ld(kdim), with row exponents rexp (A)
// and cexp (X).  R and B are n x k, column-major.
void digit_gemm(int64_t n, int64_t k, int64_t kdim, const void* Ad, int nda, const int* rexp, const void* Xd, int ndx,
                int64_t kpad, const int* cexp, int beta, int lmax, const double* B, int64_t ldb, double sgn, double* R,
                int64_t ldr, int* err, cudaStream_t s, const char* prof_name) {
    if (n <= 0 || k <= 0) return;
    if (n > (1 << 30) / 8 || kdim <= 0 || kpad < k || kpad % 16) throw Error(OMG_ERR_INVALID, "digit GEMM: bad sizes");
    ProfScope prof_(prof_name, s);
    const int64_t ld = digits_ld(kdim);
    // plan: digit pairs by level, level sums flushed before they could leave int32
    tcr::PairPlan plan{};
    const double win_bound = (double)tcr::KC * std::ldexp(1.0, 2 * beta);
    if (win_bound >= std::ldexp(1.0, 23)) throw Error(OMG_ERR_INVALID, "digit GEMM: window not exact");
    auto amax = [&](int d) { return std::ldexp(1.0, d == 1 ? beta : beta - 1); };
    std::vector<std::pair<int, int>> pairs;
    for (int lev = 2; lev <= lmax; ++lev)
        for (int a = std::max(1, lev - ndx); a <= std::min(nda, lev - 1); ++a) pairs.push_back({a, lev - a});
    if ((int)pairs.size() > tcr::MAXPAIRS) throw Error(OMG_ERR_INVALID, "digit GEMM: too many digit pairs");
    plan.n = (int)pairs.size();
    const int64_t nchunk = (kdim + tcr::BK - 1) / tcr::BK;
    plan.nwin = (int)((nchunk + tcr::CPW - 1) / tcr::CPW);
    const double lim = std::ldexp(1.0, 31) * 0.9;
    double run = 0.0;
    for (int p = 0; p < plan.n; ++p) {
        plan.s[p] = (uint8_t)pairs[p].first;
        plan.t[p] = (uint8_t)pairs[p].second;
        const double bound = (double)plan.nwin * tcr::KC * amax(pairs[p].first) * amax(pairs[p].second);
        if (bound >= lim) throw Error(OMG_ERR_UNSUPPORTED, "residual digits: matrix too large for int32 sums");
        run += bound;
        const bool last = p + 1 == plan.n;
        bool flush = last || pairs[p + 1].first + pairs[p + 1].second != pairs[p].first + pairs[p].second;
        if (!flush) {
            const double nb = (double)plan.nwin * tcr::KC * amax(pairs[p + 1].first) * amax(pairs[p + 1].second);
            flush = run + nb >= lim;
        }
        if (flush) {
            plan.flush |= 1ull << p;
            run = 0.0;
        }
    }
    if (!B)
        OMG_CUDA(cudaMemset2DAsync(R, ldr * 8, 0, n * 8, k, s));
    else if (B != R)
        OMG_CUDA(cudaMemcpy2DAsync(R, ldr * 8, B, ldb * 8, n * 8, k, cudaMemcpyDeviceToDevice, s));
    static bool attr = false;
    static int n_sm = 0;
    if (!attr) {
        cudaFuncSetAttribute(tcr::residual_slices_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tcr::SMEM_BYTES);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (n_sm <= 0) n_sm = 1;
        attr = true;
    }
    // tile width: all columns in one tile (each A digit plane streamed once per digit pair) unless that leaves
    // more than half the SMs idle; then narrower tiles (multiples of 16 columns, >= 64)
    const int nrb = (int)((n + tcr::BM - 1) / tcr::BM);
    int ncb = (int)((k + tcr::BN - 1) / tcr::BN);
    auto width = [&](int nc) { return (int)(((k + nc - 1) / nc + 15) / 16 * 16); };
    while (2 * (int64_t)nrb * ncb < n_sm && width(ncb + 1) >= 64) ++ncb;
    const int nmma = width(ncb);
    const CUtensorMap mA = tc::make_map_2d(Ad, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (int64_t)nda * n, ld, ld, tcr::BK,
                                           tcr::BM);
    const CUtensorMap mX = tc::make_map_2d(Xd, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (int64_t)ndx * kpad, ld, ld,
                                           tcr::BK, nmma);
    // few output tiles (a short side of the product): each tile's digit pairs are split into level-aligned
    // groups, contiguous runs of levels with about equal pair counts, summed into separate slices and added
    // in a fixed order afterwards (deterministic)
    std::vector<int> lbeg;
    for (int p = 0; p < plan.n; ++p)
        if (p == 0 || pairs[p].first + pairs[p].second != pairs[p - 1].first + pairs[p - 1].second) lbeg.push_back(p);
    lbeg.push_back(plan.n);
    const int nlev = (int)lbeg.size() - 1;
    const int64_t tiles = (int64_t)nrb * ncb;
    const int G = (int)std::max<int64_t>(1, std::min<int64_t>({n_sm / tiles, (int64_t)tcr::MAXGROUPS, (int64_t)nlev}));
    {   // contiguous partition of the levels into G groups minimising the largest pair count
        const int INF = 1 << 30;
        std::vector<std::vector<int>> best(G + 1, std::vector<int>(nlev + 1, INF)), cut(G + 1, std::vector<int>(nlev + 1, 0));
        best[0][0] = 0;
        for (int g = 1; g <= G; ++g)
            for (int i = g; i <= nlev; ++i)
                for (int j = g - 1; j < i; ++j) {
                    if (best[g - 1][j] == INF) continue;
                    const int c = std::max(best[g - 1][j], lbeg[i] - lbeg[j]);
                    if (c < best[g][i]) {
                        best[g][i] = c;
                        cut[g][i] = j;
                    }
                }
        plan.ngroups = G;
        int i = nlev;
        for (int g = G; g >= 1; --g) {
            plan.gbeg[g] = lbeg[i];
            i = cut[g][i];
        }
        plan.gbeg[0] = 0;
    }
    DevBuf parts(G > 1 ? (size_t)(G - 1) * n * k * 8 : 0, s);
    if (G > 1) OMG_CUDA(cudaMemsetAsync(parts.p, 0, (size_t)(G - 1) * n * k * 8, s));
    const int64_t ntiles = tiles * G;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, n_sm);
    tcr::residual_slices_kernel<<<grid, tcr::THREADS, tcr::SMEM_BYTES, s>>>(mA, mX, plan, (int)n, (int)k, (int)kpad,
                                                                            beta, rexp, cexp, sgn, R, ldr,
                                                                            parts.as<double>(), ntiles, nrb, ncb,
                                                                            nmma, err);
    check_tcr(prof_name);
    if (G > 1) {
        tcr::sum_groups_kernel<<<dim3((unsigned)std::min<int64_t>((n + 255) / 256, 1024),
                                      (unsigned)std::min<int64_t>(k, 32768)), 256, 0, s>>>(
            n, k, G - 1, parts.as<double>(), R, ldr);
        check_tcr("digit GEMM groups");
    }
}

// R = B - A X, A symmetric n x n (its digit rows are its digit columns).
void residual_slices(int64_t n, int64_t k, const void* Ad, int nda, const int* rexp, const void* Xd, int ndx,
                     int64_t kpad, const int* cexp, int beta, int lmax, const double* B, int64_t ldb, double* R,
                     int64_t ldr, int* err, cudaStream_t s) {
    digit_gemm(n, k, n, Ad, nda, rexp, Xd, ndx, kpad, cexp, beta, lmax, B, ldb, -1.0, R, ldr, err, s, "residual_tc");
}

}  // namespace omg

// Test hook (not part of the public header): R = B - A X through the digits
// and the tensor-core kernel, A symmetric n x n, X and B n x k (column-major,
// device pointers), with the solver's parameters (7 digits of 7 bits, level <= 8).
extern "C" int omg_internal_residual_tc(int64_t n, int64_t k, const double* A, const double* X, const double* B,
                                        double* R, int* err) {
    void* ad = nullptr;
    void* xd = nullptr;
    int* rexp = nullptr;
    int* cexp = nullptr;
    int rc = 0;
    try {
        const int nd = 7, beta = 7;
        const int64_t ld = omg::digits_ld(n), kpad = (k + 127) / 128 * 128;
        if (cudaMalloc(&ad, (size_t)nd * n * ld * 2) != cudaSuccess ||
            cudaMalloc(&xd, (size_t)nd * kpad * ld * 2) != cudaSuccess ||
            cudaMalloc(&rexp, (size_t)n * sizeof(int)) != cudaSuccess ||
            cudaMalloc(&cexp, (size_t)kpad * sizeof(int)) != cudaSuccess)
            throw omg::Error(OMG_ERR_NOMEM, "test hook allocation");
        omg::digits_columns(A, n, n, n, nd, beta, n, ld, ad, rexp, 0);
        omg::digits_columns(X, n, k, n, nd, beta, kpad, ld, xd, cexp, 0);
        omg::residual_slices(n, k, ad, nd, rexp, xd, nd, kpad, cexp, beta, nd + 1, B, n, R, n, err, 0);
        rc = cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        rc = e.code;
    }
    cudaFree(ad);
    cudaFree(xd);
    cudaFree(rexp);
    cudaFree(cexp);
    return rc;
}

// Test hook: the digit planes of a column-major FP64 matrix (device
// pointers): nd planes of rows_per_plane rows of ldo bf16, column exponents.
extern "C" int omg_internal_digits(const double* M, int64_t n, int64_t ncol, int64_t ldm, int nd, int beta,
                                   int64_t rows_per_plane, int64_t ldo, void* out, int* ex) {
    try {
        omg::digits_columns(M, n, ncol, ldm, nd, beta, rows_per_plane, ldo, out, ex, 0);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        return e.code;
    }
}
