// Tensor-core (tcgen05, sm_103a) grouped gather/scatter GEMM for the
// precision form's translations:  D[:, out(p), r] (+)= A_g B[:, in(p), r].
//
// Every FP32 operand is split into three bf16 terms, a = a0 + a1 + a2 (each
// term holds the next 8 significant bits), and the product is accumulated
// from the six bf16 MMAs that reach 2^-24 relative size (a0b0, a0b1, a1b0,
// a0b2, a1b1, a2b0) in FP32 accumulators in tensor memory: FP32-level
// accuracy on the bf16 tensor pipe.  The accumulation error of an FP32
// tensor-memory accumulator grows with the number of MMAs added into it, so
// the dominant product a0b0 and the five small products go to separate
// accumulators, added in FP32 registers by the epilogue: small terms are
// never rounded against the large sum.  The operators' planes are built once
// at setup; the B operand (cell coefficients) is split before every use.
//
// Persistent and warp-specialized: one CTA per SM walks the 128 x BN output
// tiles (all row tiles of a column tile back to back, so the gathered B
// columns are reused from L2).  K runs in chunks of 64 bf16 (128-byte rows)
// through a ring of shared-memory stages, each holding six 128B-swizzled
// K-major planes (three of A, three of B).
//   warps 8-11 producers: cp.async of the A rows and the B rows (gathered by
//              pair), four whole 128-byte rows per warp instruction; a stage
//              is handed over through its "full" mbarrier once the copies
//              have landed;
//   warp 12    one thread issues the chunk's 24 MMAs and commits them to the
//              stage's "empty" mbarrier (and, after a tile's last chunk, to
//              the accumulator's "full" mbarrier);
//   warps 0-7  epilogue: tcgen05.ld of the tile's two accumulators (warp w
//              owns TMEM lanes 32 (w % 4) .. + 31 and every other 32-column
//              chunk, from chunk w / 4), scatter into D, release the
//              accumulator.  Two accumulator buffers let a tile's epilogue
//              overlap the next tile's MMAs; eight warps rather than four
//              made the M2L launch 11 % shorter (the tile's TMEM reads and
//              scattered adds had been pacing the MMAs).
// Every wait is bounded; a timed-out wait raises a CTA-wide abort flag that
// ends every role's loop, the MMAs in flight are drained (bounded) before
// tensor memory is freed, and the kernel reports through the error flag.
#include <cuda_bf16.h>
#include <stdint.h>

#include "plan.h"

namespace tbem {

constexpr int TC_BM = 128, TC_BK = 64;                       // TC_BK: the planes' K padding
constexpr int TC_TERMS = 3;                                  // bf16 terms per operand
constexpr long long TC_WAIT_CYCLES = 4000000000LL;          // ~2 s at 2 GHz

// Tile shapes (the autotuner picks one per operator set): N = 128 columns and
// 64-deep K chunks (128-byte rows, 128B swizzle) in a 2-stage ring; N = 64,
// 64-deep, 3 stages; N = 128 with 32-deep chunks (64-byte rows, 64B swizzle)
// in a 4-stage ring, which keeps three chunks in flight; N = 256, 32-deep,
// 3 stages (each A chunk serves twice the columns: less shared-memory
// traffic per MMA), one accumulator buffer.
template <int BN, int BK>
struct TcShape {
    static_assert(BK == 64 || BK == 32, "K chunk");
    static constexpr int RB = BK * 2;                                     // bytes per tile row
    static constexpr int STAGES = BK == 32 ? (BN == 256 ? 3 : 4) : (BN == 128 ? 2 : 3);
    static constexpr int A_TILE = TC_BM * RB;                             // one A plane tile
    static constexpr int B_TILE = BN * RB;                                // one B plane tile
    static constexpr int STAGE_BYTES = TC_TERMS * (A_TILE + B_TILE);
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
    // accumulator buffers of (big, small): two while they fit in the 512
    // tensor-memory columns (the epilogue overlaps the next tile), else one
    static constexpr int NBUF = 4 * BN <= 512 ? 2 : 1;
    static constexpr uint32_t TMEM_COLS = NBUF * 2 * BN;
    // kind::f16, bf16 A/B, FP32 D, K-major A and B, M = 128, N = BN
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) |
                                      ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
};
static_assert(TcShape<128, 64>::SMEM_BYTES <= 227 * 1024 && TcShape<64, 64>::SMEM_BYTES <= 227 * 1024 &&
                  TcShape<128, 32>::SMEM_BYTES <= 227 * 1024 && TcShape<256, 32>::SMEM_BYTES <= 227 * 1024,
              "shared memory budget");
static_assert(TcShape<256, 32>::TMEM_COLS == 512 && TcShape<128, 64>::TMEM_COLS == 512, "tensor memory");
constexpr int TC_PRODUCERS = 128;                      // producer threads (warps 4-7)
constexpr int TC_EPILOGUE = 256;                     // epilogue threads (warps 0-7)
constexpr int TC_THREADS_P = TC_EPILOGUE + TC_PRODUCERS + 32;  // epilogue + producers + MMA warp

struct TcArgs {
    const __nv_bfloat16* A[TC_TERMS];  // [op][m_pad][k_pad] per term
    long a_op_stride;                  // m_pad * k_pad
    int k_pad;
    // per column tile: {operator, first pair of its group, first column of
    // the tile within the group, columns of the group}; column c of a group
    // is (pair pair0 + c / nrhs, right-hand side c % nrhs), its B row
    // in_cell[pair] * nrhs + rhs and its D column out_cell[pair] * nrhs + rhs
    const int4* tiles;
    // when they fit: every column's B row and D column precomputed per tile
    // ([tile][BN], -1 past the end), one load with no division; else null
    const int* tile_brow;
    const int* tile_drow;
    const int* in_cell;
    const int* out_cell;
    int nrhs;
    const __nv_bfloat16* B[TC_TERMS];  // [cell][rhs][k_pad] per term
    float* D;                          // [cell][rhs][n]
    int n;
    int atomic;
    int* err;
    long long wait_cycles;             // budget of every role's bounded wait
};

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: K-major rows of RB bytes with the RB-byte
// swizzle (128 or 64), 8-row groups 8 * RB bytes apart.
template <int RB>
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused with a swizzle)
    d |= (uint64_t)((8 * RB) >> 4) << 32;    // stride byte offset
    d |= (uint64_t)1 << 46;                  // descriptor version
    d |= (uint64_t)(RB == 128 ? 2 : 4) << 61;  // SWIZZLE_128B / SWIZZLE_64B
    return d;
}

// Position of 16-byte piece j of tile row r under the RB-byte swizzle: the
// piece index XOR the row's position inside the 1024-byte (128B) or
// 512-byte (64B) swizzle atom.
template <int RB>
__device__ __forceinline__ uint32_t sw_piece(int row, int j)
{
    return RB == 128 ? (uint32_t)(j ^ (row & 7)) : (uint32_t)(j ^ ((row >> 1) & 3));
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accum)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false if the phase did not complete within the budget.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    long long t0 = clock64();
    while (!mbar_try(mbar, parity)) {
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    }
    return true;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

template <int BN, int BK>
__global__ void __launch_bounds__(TC_THREADS_P, 1) tc_gemm_kernel(const TcArgs a, int n_ctiles, int m_tiles)
{
    using Sh = TcShape<BN, BK>;
    constexpr int RB = Sh::RB;
    constexpr int STAGES = Sh::STAGES;
    constexpr int LAG = STAGES - 1;  // chunks a producer keeps in flight before a hand-over
    static_assert(LAG >= 1 && LAG <= 3, "stage count");
    constexpr int B_BASE = TC_TERMS * Sh::A_TILE;  // B planes follow the A planes
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accf_bar[2], acce_bar[2], drain_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int nk = a.k_pad / BK;
    const int total = n_ctiles * m_tiles;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_slot)),
                     "r"(Sh::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_bar[s])), "r"(TC_PRODUCERS));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[s])));
        }
        for (int b = 0; b < 2; b++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&accf_bar[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acce_bar[b])), "r"(TC_EPILOGUE));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&drain_bar)));
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t smem0 = smem_u32(smem);

    // bounded wait that also gives up as soon as another role aborted
    auto wait = [&](uint64_t* bar, uint32_t parity) -> bool {
        const uint32_t b = smem_u32(bar);
        const long long t0 = clock64();
        while (!mbar_try(b, parity)) {
            if (*reinterpret_cast<volatile int*>(&abort_flag)) return false;
            if (clock64() - t0 > a.wait_cycles) {
                atomicExch(&abort_flag, 1);
                return false;
            }
        }
        return true;
    };

    bool mma_issued = false;
    if (warp >= 8 && warp < 12) {
        // ---------------- producers.  A plane tile is 128 rows of PPR 16-byte
        // pieces; piece e = pt + 128 i is row e / PPR, piece e % PPR, so one
        // warp instruction copies whole rows (full sectors, coalesced).
        constexpr int PPR = RB / 16;                       // pieces per row (8 or 4)
        constexpr int RSTEP = TC_PRODUCERS / PPR;          // rows between a thread's pieces
        constexpr int A_PER = TC_BM / RSTEP;               // pieces of A per thread and plane
        constexpr int B_PER = BN / RSTEP;                  // pieces of B per thread and plane
        const int pt = tid - TC_EPILOGUE;
        const int pj = pt % PPR, prow = pt / PPR;  // piece within a row; rows prow + RSTEP i
        // the next tile's operator and B rows, loaded one tile ahead (plain
        // independent loads: their latency hides behind the current tile)
        int nop = 0, nb[B_PER];
        auto prefetch = [&](int t) {
            const int tile = t / m_tiles;
            const int4 ti = a.tiles[tile];
            nop = ti.x;
            if (a.tile_brow) {
#pragma unroll
                for (int i = 0; i < B_PER; i++) nb[i] = a.tile_brow[(long)tile * BN + prow + RSTEP * i];
            } else {
#pragma unroll
                for (int i = 0; i < B_PER; i++) {
                    const int c = ti.z + prow + RSTEP * i;
                    nb[i] = c < ti.w ? a.in_cell[ti.y + c / a.nrhs] * a.nrhs + c % a.nrhs : -1;
                }
            }
        };
        if (blockIdx.x < total) prefetch(blockIdx.x);
        int j = 0;  // chunks issued (over all tiles of this CTA)
        bool ok = true;
        for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
            const int m0 = (t % m_tiles) * TC_BM;
            const long a_base = (long)nop * a.a_op_stride + (long)(m0 + prow) * a.k_pad + pj * 8;
            long boff[B_PER];
#pragma unroll
            for (int i = 0; i < B_PER; i++) boff[i] = nb[i] >= 0 ? (long)nb[i] * a.k_pad + pj * 8 : -1;
            if (t + (int)gridDim.x < total) prefetch(t + gridDim.x);
            for (int kc = 0; kc < nk; kc++, j++) {
                const int s = j % STAGES;
                if (j >= STAGES && !wait(&empty_bar[s], ((j / STAGES) - 1) & 1)) {
                    ok = false;
                    break;
                }
                const uint32_t st = smem0 + s * Sh::STAGE_BYTES;
                const int k0 = kc * BK;
#pragma unroll
                for (int q = 0; q < TC_TERMS; q++) {
#pragma unroll
                    for (int i = 0; i < A_PER; i++) {
                        const int row = prow + RSTEP * i;
                        const uint32_t dst = st + q * Sh::A_TILE + row * RB + (sw_piece<RB>(row, pj) << 4);
                        const __nv_bfloat16* src = a.A[q] + a_base + (long)RSTEP * i * a.k_pad + k0;
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
                    }
#pragma unroll
                    for (int i = 0; i < B_PER; i++) {
                        const int row = prow + RSTEP * i;
                        const uint32_t dst = st + B_BASE + q * Sh::B_TILE + row * RB + (sw_piece<RB>(row, pj) << 4);
                        const bool v = boff[i] >= 0;
                        // an invalid column is zero-filled (source size 0, nothing read)
                        const __nv_bfloat16* src = v ? a.B[q] + boff[i] + k0 : a.B[q];
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src),
                                     "r"(v ? 16u : 0u)
                                     : "memory");
                    }
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
                if (j >= LAG) {
                    // chunk j - LAG has landed: hand its stage over (LAG chunks
                    // stay in flight behind it)
                    if constexpr (LAG == 1) asm volatile("cp.async.wait_group 1;" ::: "memory");
                    else if constexpr (LAG == 2) asm volatile("cp.async.wait_group 2;" ::: "memory");
                    else asm volatile("cp.async.wait_group 3;" ::: "memory");
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_arrive(smem_u32(&full_bar[(j - LAG) % STAGES]));
                }
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (ok) {
            // hand over the chunks still held back
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (int q = max(0, j - LAG); q < j; q++) mbar_arrive(smem_u32(&full_bar[q % STAGES]));
        }
    } else if (warp == 12) {
        // ---------------- MMA issue (one thread)
        if (lane == 0) {
            int j = 0, tc = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < total && ok; t += gridDim.x, tc++) {
                const int b = tc % Sh::NBUF, bu = tc / Sh::NBUF;
                if (bu >= 1 && !wait(&acce_bar[b], (bu - 1) & 1)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t big = tmem + b * 2 * BN, small = big + BN;
                for (int kc = 0; kc < nk; kc++, j++) {
                    const int s = j % STAGES;
                    if (!wait(&full_bar[s], (j / STAGES) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t st = smem0 + s * Sh::STAGE_BYTES;
#pragma unroll
                    for (int kk = 0; kk < BK / 16; kk++) {
                        const uint32_t off = kk * 32;  // 16 bf16 along K inside the swizzle atom
                        const uint32_t a0 = st + off, a1 = a0 + Sh::A_TILE, a2 = a0 + 2 * Sh::A_TILE;
                        const uint32_t b0 = st + B_BASE + off, b1 = b0 + Sh::B_TILE, b2 = b0 + 2 * Sh::B_TILE;
                        constexpr uint32_t ID = Sh::IDESC;
                        const uint32_t acc = (kc | kk) != 0;
                        mma_bf16(big, sw_desc<RB>(a0), sw_desc<RB>(b0), ID, acc);
                        mma_bf16(small, sw_desc<RB>(a0), sw_desc<RB>(b1), ID, acc);
                        mma_bf16(small, sw_desc<RB>(a1), sw_desc<RB>(b0), ID, 1);
                        mma_bf16(small, sw_desc<RB>(a0), sw_desc<RB>(b2), ID, 1);
                        mma_bf16(small, sw_desc<RB>(a1), sw_desc<RB>(b1), ID, 1);
                        mma_bf16(small, sw_desc<RB>(a2), sw_desc<RB>(b0), ID, 1);
                    }
                    mma_issued = true;
                    mma_commit(smem_u32(&empty_bar[s]));
                }
                if (!ok) break;
                mma_commit(smem_u32(&accf_bar[b]));
            }
        }
    } else {
        // ---------------- epilogue (warps 0-7)
        constexpr int NCC = BN / 32;
        int tc = 0;
        for (int t = blockIdx.x; t < total; t += gridDim.x, tc++) {
            const int b = tc % Sh::NBUF, bu = tc / Sh::NBUF;
            const int m0 = (t % m_tiles) * TC_BM;
            // lane q of a 32-column chunk resolves column q's destination; the
            // loads overlap the wait for the accumulator
            const int tile = t / m_tiles;
            int drow[NCC];
            if (a.tile_drow) {
#pragma unroll
                for (int cc = 0; cc < NCC; cc++) drow[cc] = a.tile_drow[(long)tile * BN + cc * 32 + lane];
            } else {
                const int4 ti = a.tiles[tile];
#pragma unroll
                for (int cc = 0; cc < NCC; cc++) {
                    const int c = ti.z + cc * 32 + lane;
                    drow[cc] = c < ti.w ? a.out_cell[ti.y + c / a.nrhs] * a.nrhs + c % a.nrhs : -1;
                }
            }
            if (!wait(&accf_bar[b], bu & 1)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int row = m0 + (warp % 4) * 32 + lane;
#pragma unroll
            for (int cc = warp / 4; cc < NCC; cc += 2) {
                float v[32], w[32];
                const uint32_t lane_base = tmem + ((uint32_t)((warp % 4) * 32) << 16) + b * 2 * BN + cc * 32;
                const long my_off = drow[cc] >= 0 ? (long)drow[cc] * a.n : -1;
                tmem_ld32(lane_base + BN, v);  // small terms first
                tmem_ld32(lane_base, w);
#pragma unroll
                for (int q = 0; q < 32; q++) v[q] += w[q];
#pragma unroll
                for (int q = 0; q < 32; q++) {
                    const long off = __shfl_sync(0xffffffffu, my_off, q);
                    if (off >= 0 && row < a.n) {
                        float* dst = a.D + off + row;
                        if (a.atomic) atomicAdd(dst, v[q]);
                        else *dst += v[q];
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(smem_u32(&acce_bar[b]));
        }
    }
    __syncthreads();
    // drain: every MMA this CTA issued has completed before tensor memory is
    // released (bounded by the fixed default budget, never by a shortened
    // one: after an abort the MMAs in flight still finish)
    if (warp == 12 && lane == 0 && mma_issued) {
        mma_commit(smem_u32(&drain_bar));
        if (!mbar_wait(smem_u32(&drain_bar), 0)) atomicExch(&abort_flag, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && abort_flag) atomicExch(a.err, 1);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Sh::TMEM_COLS));
}

// v -> three bf16 terms t0 + t1 + t2 (each the rounding of what is left)
__device__ __forceinline__ void split3(float v, __nv_bfloat16& t0, __nv_bfloat16& t1,
                                       __nv_bfloat16& t2)
{
    t0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(t0);
    t1 = __float2bfloat16_rn(r1);
    t2 = __float2bfloat16_rn(r1 - __bfloat162float(t1));
}

// in [rows][n] FP32 -> three bf16 planes [rows][k_pad] (columns >= n zero)
__global__ void split_rows_kernel(const float* in, long rows, int n, int k_pad,
                                  __nv_bfloat16* o0, __nv_bfloat16* o1, __nv_bfloat16* o2)
{
    const long total = rows * k_pad;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long r = t / k_pad;
        const int k = (int)(t % k_pad);
        split3(k < n ? in[r * n + k] : 0.f, o0[t], o1[t], o2[t]);
    }
}

// operators [op][m][k] FP32 -> three bf16 planes [op][m_pad][k_pad] (zero padding)
__global__ void split_ops_kernel(const float* in, long n_ops, int m, int k, int m_pad, int k_pad,
                                 __nv_bfloat16* o0, __nv_bfloat16* o1, __nv_bfloat16* o2)
{
    const long total = n_ops * m_pad * (long)k_pad;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const int kk = (int)(t % k_pad);
        const long rm = t / k_pad;
        const int mm = (int)(rm % m_pad);
        const long op = rm / m_pad;
        split3((mm < m && kk < k) ? in[(op * m + mm) * (long)k + kk] : 0.f, o0[t], o1[t], o2[t]);
    }
}

}  // namespace

void TcPlanes::build(const float* ops32, long n_ops, int m, int k, cudaStream_t s)
{
    this->m = m;
    this->k = k;
    m_pad = (m + TC_BM - 1) / TC_BM * TC_BM;
    k_pad = (k + TC_BK - 1) / TC_BK * TC_BK;
    const long total = n_ops * (long)m_pad * k_pad;
    for (auto& p : a) p.alloc(std::max<long>(total, 1));
    if (total > 0) {
        split_ops_kernel<<<(unsigned)std::min<long>((total + 255) / 256, 152L * 64), 256, 0, s>>>(
            ops32, n_ops, m, k, m_pad, k_pad, a[0].p, a[1].p, a[2].p);
        TBEM_CK(cudaGetLastError());
    }
    err.alloc(1);
    TBEM_CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    // per device: set on every build (the plan's device is current)
    TBEM_CK(cudaFuncSetAttribute(tc_gemm_kernel<128, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<128, 64>::SMEM_BYTES));
    TBEM_CK(cudaFuncSetAttribute(tc_gemm_kernel<64, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<64, 64>::SMEM_BYTES));
    TBEM_CK(cudaFuncSetAttribute(tc_gemm_kernel<128, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<128, 32>::SMEM_BYTES));
    TBEM_CK(cudaFuncSetAttribute(tc_gemm_kernel<256, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<256, 32>::SMEM_BYTES));
}

void TcPlanes::split_b(const float* cells, long rows, cudaStream_t s)
{
    const long total = rows * (long)k_pad;
    for (auto& p : b) p.ensure(std::max<long>(total, 1));
    if (total > 0) {
        split_rows_kernel<<<(unsigned)std::min<long>((total + 255) / 256, 152L * 64), 256, 0, s>>>(
            cells, rows, k, k_pad, b[0].p, b[1].p, b[2].p);
        TBEM_CK(cudaGetLastError());
    }
}

void TcPlanes::split_b_rows(const float* cells, long row0, long rows, long rows_total,
                            cudaStream_t s)
{
    for (auto& p : b) p.ensure(std::max<long>(rows_total * (long)k_pad, 1));
    const long total = rows * (long)k_pad;
    if (total > 0) {
        split_rows_kernel<<<(unsigned)std::min<long>((total + 255) / 256, 152L * 64), 256, 0, s>>>(
            cells + row0 * (long)k, rows, k, k_pad, b[0].p + row0 * k_pad, b[1].p + row0 * k_pad,
            b[2].p + row0 * k_pad);
        TBEM_CK(cudaGetLastError());
    }
}

void GemmSet::run_tc(const TcPlanes& P, float* D, int nrhs, int atomic, long nn, cudaStream_t s,
                     long* launches)
{
    if (empty()) return;
    const int bn = tc_bn == 64 ? 64 : tc_bn == 256 ? 256 : 128;
    const int key = nrhs * 1024 + bn;
    auto it = tc_tiles.find(key);
    if (it == tc_tiles.end()) {
        // column tiles of every group: (operator, group's first pair, first
        // column, the group's column count)
        std::vector<int4> t;
        for (size_t g = 0; g < npairs.size(); g++) {
            const long ncols = (long)npairs[g] * nrhs;
            if (ncols > INT32_MAX || pair0[g] > INT32_MAX)
                throw Error(TBEM_ERR_ARG, "tensor-core GEMM group too large");
            for (long c = 0; c < ncols; c += bn)
                t.push_back(make_int4((int)(A_off[g] / nn), (int)pair0[g], (int)c, (int)ncols));
        }
        if (t.size() > (size_t)INT32_MAX / 4) throw Error(TBEM_ERR_ARG, "too many tensor-core tiles");
        TcTiles& e = tc_tiles[key];
        e.t.upload(t);
        e.n = (int)t.size();
        // per-column rows as well while they stay small (up to 2^25 columns,
        // 128 MB per table): the kernel then reads each column's row directly
        if (t.size() * bn <= (size_t(1) << 25)) {
            std::vector<int> brow(t.size() * bn), drow(t.size() * bn);
            for (size_t i = 0; i < t.size(); i++)
                for (int jj = 0; jj < bn; jj++) {
                    const int c = t[i].z + jj;
                    const bool v = c < t[i].w;
                    const long p = t[i].y + c / nrhs;
                    brow[i * bn + jj] = v ? in_cell[p] * nrhs + c % nrhs : -1;
                    drow[i * bn + jj] = v ? out_cell[p] * nrhs + c % nrhs : -1;
                }
            e.brow.upload(brow);
            e.drow.upload(drow);
        }
        it = tc_tiles.find(key);
    }
    TcArgs a;
    for (int t = 0; t < TC_TERMS; t++) {
        a.A[t] = P.a[t].p;
        a.B[t] = P.b[t].p;
    }
    a.a_op_stride = (long)P.m_pad * P.k_pad;
    a.k_pad = P.k_pad;
    a.tiles = it->second.t.p;
    a.tile_brow = it->second.brow.p;
    a.tile_drow = it->second.drow.p;
    a.in_cell = d_in.p;
    a.out_cell = d_out.p;
    a.nrhs = nrhs;
    a.D = D;
    a.n = P.m;
    a.atomic = atomic;
    a.err = P.err.p;
    a.wait_cycles = P.wait_cycles > 0 ? P.wait_cycles : TC_WAIT_CYCLES;
    const int n_ctiles = it->second.n, m_tiles = P.m_pad / TC_BM;
    const long total = (long)n_ctiles * m_tiles;
    if (total == 0) return;
    int dev = 0, sms = 0;
    TBEM_CK(cudaGetDevice(&dev));
    TBEM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::min<long>(total, std::max(sms, 1));
    if (bn == 64)
        tc_gemm_kernel<64, 64><<<grid, TC_THREADS_P, TcShape<64, 64>::SMEM_BYTES, s>>>(a, n_ctiles, m_tiles);
    else if (bn == 256)
        tc_gemm_kernel<256, 32><<<grid, TC_THREADS_P, TcShape<256, 32>::SMEM_BYTES, s>>>(a, n_ctiles, m_tiles);
    else if (tc_bk == 32)
        tc_gemm_kernel<128, 32><<<grid, TC_THREADS_P, TcShape<128, 32>::SMEM_BYTES, s>>>(a, n_ctiles, m_tiles);
    else
        tc_gemm_kernel<128, 64><<<grid, TC_THREADS_P, TcShape<128, 64>::SMEM_BYTES, s>>>(a, n_ctiles, m_tiles);
    TBEM_CK(cudaGetLastError());
    if (launches) (*launches)++;
}

}  // namespace tbem
