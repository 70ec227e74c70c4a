// grt_ksum_tc.cuh -- the wavenumber integration on the tensor cores (tcgen05).
//
// For every output column c (get_int_val_single / _tensor, green.cu:1558-1716)
//   S_c(w, r) = sum_{t in c} coef_t r^-rpow_t D_{p(t)}(w, r),
//   D_p(w, r) = sum_k K_{q_p}(w, k) * w_k k^kp_p J_{b_p}(k r),
// one GEMM per pair p = (coefficient column q, power of k, Bessel function);
// the terms that share a pair differ only by a receiver-dependent factor,
// applied when the accumulators are drained.  The pairs are grouped by q, so
// that one MMA multiplies the coefficient tile of q by the Bessel operands of
// all its pairs at once (N = 32 receivers x pairs of q).
//
// Work division (make_tcplan): the coefficient columns are dealt into two
// groups of about equal pair counts (even and odd CTAs of one launch); a CTA
// owns 64 frequencies (M = 128 rows: real parts in rows 0-63, imaginary
// parts in rows 64-127), 32 receivers, one group and a slice of the k range
// (split-K).  The accumulators of the group's pairs live in tensor memory
// (pairs x 32 columns).  Halving the pairs per CTA doubles the receivers an
// operand tile is multiplied with: shared-memory traffic per multiply-add
// (operand copies, tensor-core reads, Bessel-operand stores), the limit of the
// earlier 16-receiver form, falls by 40 %.
//
// Precision: 3xTF32 -- each FP32 operand x is split into hi = tf32(x) and
// lo = tf32(x - hi) and the product is hi*hi + hi*lo + lo*hi with FP32
// accumulation (about 2^-21 relative per product).  Partial sums of the k
// slices and of the two groups are added with TwoSum by ksum_tc_reduce_kernel.
//
// Roles (320 threads): warps 0-7 produce the Bessel operand tiles in shared
// memory (canonical K-major layout, no swizzle: 8-row x 16-byte core
// matrices), one (receiver, k) of a stage per thread, and drain the
// accumulators at the end (warps w and w + 4 share a quarter of the
// tensor-memory lanes and split the output columns); one thread of warp 8
// issues the bulk copies of the coefficient tiles and raw Bessel rows up to
// SA stages ahead (the copy ring, TcRing); warp 9 allocates tensor memory and
// one of its threads issues tcgen05.mma and tcgen05.commit.  A copy slot is
// guarded by "land" (coefficient copy), "raw" (Bessel copy) and "empty"
// (MMAs done) mbarriers, an operand slot by "full" (producers) and "bempty"
// (MMAs done).  Every wait is bounded: on timeout the CTA records an error,
// skips to the end, waits (bounded) for its copies in flight and still frees
// its tensor memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "grt_integrate.cuh"
#include "grt_types.h"

namespace grt {

namespace tc {

constexpr int kM = 128;        // rows: 64 frequencies x (re, im)
constexpr int kW = 64;         // frequencies per CTA
constexpr int kN = 32;         // receivers per CTA
constexpr int kKT = 8;         // k per stage of the 3xTF32 form = one tf32 MMA K (the granularity of k slices)
constexpr int kProdWarps = 8;  // 32 receivers x 8 k pairs... one (receiver, k group) per thread
constexpr int kProducers = 32 * kProdWarps;
constexpr int kCopyWarp = kProdWarps, kMmaWarp = kProdWarps + 1;
constexpr int kThreads = kProducers + 64;
constexpr int kCoreBytes = 128;                      // 8 rows x 16 bytes
constexpr int kATileBytes = (kM / 8) * 2 * kCoreBytes;   // 4096: one q, one split (2 core matrices along K)
constexpr int kBTileBytes = (kN / 8) * 2 * kCoreBytes;   // 1024: one pair, one split
constexpr uint32_t kTmemCols = 512;
static_assert(kN == kBesselTile, "a CTA's receivers are one tile of the Bessel table");

// The two split-precision forms.  3xTF32: 8 k per stage (a row of a tile is 8
// tf32 = 32 bytes), one (receiver, k) per producer.  3xBF16: 16 k per stage
// (16 bf16 = 32 bytes), two consecutive k per producer (their bf16 words
// packed in one store; the raw Bessel rows of a stage double).
enum TcForm { kTF32 = 0, kBF16 = 1 };
template <int PREC> struct TcPrec;
template <> struct TcPrec<kTF32> { static constexpr int KT = 8, KPT = 1; };
template <> struct TcPrec<kBF16> { static constexpr int KT = 16, KPT = 2; };
template <int PREC> constexpr int raw_bytes() { return TcPrec<PREC>::KT * NBASIS * kN * 4; }
static_assert(kProducers * TcPrec<kTF32>::KPT == kN * TcPrec<kTF32>::KT, "producers cover a stage");
static_assert(kProducers * TcPrec<kBF16>::KPT == kN * TcPrec<kBF16>::KT, "producers cover a stage");

// one group of a column layout's tensor-core plan
template <int SRC, int GRP, int PREC> struct TcGroup {
    static constexpr TcPlan P = make_tcplan<SRC>();
    static constexpr int NQ = P.gnq[GRP];     // operand tiles (coefficient columns)
    static constexpr int NP = P.gnp[GRP];     // pairs
    static constexpr int Q0 = P.gq0[GRP];     // first tile in a stage block
    static constexpr int NQU = P.nqu;         // tiles in a stage block (both groups)
    static constexpr int kABytes = NQ * 2 * kATileBytes;
    static constexpr int kBBytes = NP * 2 * kBTileBytes;
    static constexpr int kRawBytes = raw_bytes<PREC>();
    static constexpr int kASlotBytes = kABytes + kRawBytes;   // a slot of the copy ring
    static_assert(NP * kN <= (int)kTmemCols, "accumulators exceed tensor memory");
    static_assert(kASlotBytes % 1024 == 0 && kBBytes % 1024 == 0, "slots stay 1024-byte aligned");
};

// Two rings of shared-memory slots.  The copy ring (SA slots) holds what the
// bulk copies bring: the coefficient tiles and the raw Bessel rows of a
// stage, issued up to SA stages ahead of the MMAs.  The operand ring (SB = 2
// slots) holds the Bessel operand the producers form from the raw rows just
// before its MMAs.  Only the copies need the depth (their latency is the
// long one), so SA is as large as shared memory allows: 4 for the moment
// tensor's 3xTF32 sums (3 shared stages before), 3 elsewhere.
constexpr int kSmemBudget = 232448 - 2048 - 1024;   // the opt-in limit less static data and alignment
#ifndef TC_OPERAND_SLOTS
#define TC_OPERAND_SLOTS 2
#endif
template <int SRC, int PREC> struct TcRing {
    static constexpr int need(int sa, int sb, int g)
    {
        return g == 0 ? sa * TcGroup<SRC, 0, PREC>::kASlotBytes + sb * TcGroup<SRC, 0, PREC>::kBBytes
                      : sa * TcGroup<SRC, 1, PREC>::kASlotBytes + sb * TcGroup<SRC, 1, PREC>::kBBytes;
    }
    static constexpr int need2(int sa, int sb) { return need(sa, sb, 0) > need(sa, sb, 1) ? need(sa, sb, 0) : need(sa, sb, 1); }
    static constexpr int SB = TC_OPERAND_SLOTS;
    static constexpr int SA = need2(4, SB) <= kSmemBudget ? 4 : need2(3, SB) <= kSmemBudget ? 3 : 2;
    static constexpr int bytes = need2(SA, SB);
    static_assert(bytes <= kSmemBudget, "the rings exceed shared memory");
};
constexpr int kMaxASlots = 4, kMaxBSlots = 3;

template <int SRC, int PREC> constexpr int smem_bytes() { return TcRing<SRC, PREC>::bytes + 1024; }

static_assert(kKT == kTileK && kM == kTileRows, "tile shape shared with the GRT kernel");
static_assert(TcPrec<kBF16>::KT == kTileK16, "tile shape shared with the GRT kernel");
template <int PREC> __device__ __forceinline__ uint32_t tile_off(int row, int k)
{
    return PREC == kBF16 ? kt_tile_off16(row, k) : kt_tile_off(row, k);
}

// shared-memory matrix descriptor: K-major, no swizzle.  LBO = distance of
// core matrices adjacent in K (128 B), SBO = distance of 8-row groups (two
// core matrices along K in both forms).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    const uint64_t lbo = kCoreBytes, sbo = 2 * kCoreBytes;
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(lbo >> 4) << 16;
    d |= (uint64_t)(sbo >> 4) << 32;
    d |= (uint64_t)1 << 46;       // descriptor version for sm_100-family tensor cores
    return d;                     // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor: dense, D = F32, A = B = TF32 (kind::tf32, format 2)
// or BF16 (kind::f16, format 1), both K-major, M = 128, N = n
template <int PREC> constexpr uint32_t idesc_n(int n)
{
    constexpr uint32_t fmt = PREC == kBF16 ? 1u : 2u;
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ float tf32_rna(float x) { return grt::tf32_rna(x); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// bulk copy global -> shared, completion on an mbarrier (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// bounded wait; false after 2^22 polls (a stage takes about a microsecond)
__device__ __forceinline__ bool mbar_wait_b(uint32_t bar, uint32_t parity)
{
    for (int it = 0; it < (1 << 22); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
// A = B = BF16 (kind::f16), D = F32
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
template <int PREC>
__device__ __forceinline__ void mma_split(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    if constexpr (PREC == kBF16) mma_bf16(dtmem, adesc, bdesc, idesc, acc);
    else mma_tf32(dtmem, adesc, bdesc, idesc, acc);
}
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// the Bessel basis functions a group uses, as a bit mask (evaluated at compile time)
#pragma nv_diagnostic push
#pragma nv_diag_suppress 20091
template <int SRC, int GRP> __host__ __device__ constexpr unsigned group_basis_mask()
{
    const TcPlan T = make_tcplan<SRC>();
    unsigned m = 0;
    for (int s = 0; s < T.gnp[GRP]; s++) {
        const int p = T.gpair[GRP][s];
        m |= 1u << Cols<SRC>::pair(p).b;
    }
    return m;
}
#pragma nv_diagnostic pop

}  // namespace tc

template <typename R>
struct KsumTcArgs {
    const float *Kt;         // operand blocks written by the GRT kernel (see GrtArgs::Kt)
    const long long *kt_base;
    const float *B;          // [nbrow][NBASIS][nr], row i at k = i dk; or tiled (bt_rows > 0)
    int bt_rows;             // > 0: B is [nr / 32][bt_rows][NBASIS][32] (unit strides only, btab_index)
    const int *nk;           // [nw]
    const int *ks;           // [nw] k stride, constant on each tile of kW frequencies (null: 1)
    const long long *koff;   // [nw]
    const double *dist;      // [nr]
    float *P;                // partial sums [nsplit][2 groups][nr][nc][nw] complex
    long long nkw;
    double dk;
    int nw, nr, nkmax, nsplit, kslice;   // kslice: k per split (multiple of kKT)
    unsigned int *err;
};

// One CTA of column group GRP; blk = (frequency tile, receiver tile, k slice).
template <int SRC, int GRP, int PREC>
__device__ __forceinline__ void ksum_tc_cta(const KsumTcArgs<float> &A, int blk, unsigned char *smem_tc,
                                            unsigned long long *bars, float *ir_s)
{
    using namespace tc;
    using CT = Cols<SRC>;
    using TG = TcGroup<SRC, GRP, PREC>;
    constexpr int NC = CT::NC, NQ = TG::NQ, NP = TG::NP;
    constexpr int KT = TcPrec<PREC>::KT, KPT = TcPrec<PREC>::KPT;
    constexpr int SA = TcRing<SRC, PREC>::SA, SB = TcRing<SRC, PREC>::SB;
    constexpr TcPlan TP = make_tcplan<SRC>();
    constexpr unsigned kBasis = group_basis_mask<SRC, GRP>();
    __shared__ uint32_t tmem_base_s;
    __shared__ int fail_s;

    const int nrt = (A.nr + kN - 1) / kN;
    const int wt = blk / (nrt * A.nsplit);
    const int rem = blk % (nrt * A.nsplit);
    const int rt = rem / A.nsplit, sp = rem % A.nsplit;
    const int w0 = wt * kW, r0 = rt * kN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // k range of this CTA: [kb, ke) within the longest frequency of the tile
    int nkt = 0;
    for (int i = 0; i < kW; i++)
        if (w0 + i < A.nw) nkt = max(nkt, A.nk[w0 + i]);
    const int kb = sp * A.kslice;
    const int ke = min(nkt, kb + A.kslice);
    const int nstage = ke > kb ? (ke - kb + KT - 1) / KT : 0;

    unsigned char *sm = (unsigned char *)(((uintptr_t)smem_tc + 1023) & ~(uintptr_t)1023);
    const uint32_t sm_s = (uint32_t)__cvta_generic_to_shared(sm);
    auto bar_at = [&](int i) { return (uint32_t)__cvta_generic_to_shared(&bars[i]); };
    // copy ring slot a: land (coefficient tiles copied), raw (Bessel rows
    // copied), empty (the MMAs that read it are done); operand ring slot b:
    // full (the producers' Bessel operand written), bempty (its MMAs done)
    auto land_bar = [&](int a) { return bar_at(a); };
    auto raw_bar = [&](int a) { return bar_at(SA + a); };
    auto empty_bar = [&](int a) { return bar_at(2 * SA + a); };
    auto full_bar = [&](int b) { return bar_at(3 * SA + b); };
    auto bempty_bar = [&](int b) { return bar_at(3 * SA + SB + b); };
    const uint32_t done_bar = bar_at(3 * SA + 2 * SB);
    const bool tiled = A.bt_rows > 0;
    // copy slot a: [A: NQ x (hi, lo) tiles][raw Bessel rows]; after the SA
    // copy slots, operand slot b: [B: (hi | lo) x NP tiles]
    auto a_tile = [&](int a, int i, int split) {
        return (uint32_t)(a * TG::kASlotBytes + (i * 2 + split) * kATileBytes);
    };
    auto raw_off = [&](int a) { return (uint32_t)(a * TG::kASlotBytes + TG::kABytes); };
    auto b_tile = [&](int b, int slot, int split) {
        return (uint32_t)(SA * TG::kASlotBytes + b * TG::kBBytes + (split * NP + slot) * kBTileBytes);
    };

    if (threadIdx.x == 0) {
        for (int a = 0; a < SA; a++) {
            tc::mbar_init(land_bar(a), 1);
            tc::mbar_init(raw_bar(a), 1);
            tc::mbar_init(empty_bar(a), 1);
        }
        for (int b = 0; b < SB; b++) {
            tc::mbar_init(full_bar(b), kProdWarps);   // one arrival per producer warp
            tc::mbar_init(bempty_bar(b), 1);
        }
        tc::mbar_init(done_bar, 1);
        fail_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // receiver factors r^-1, r^-2 of the drain's terms
    if (threadIdx.x < kN) {
        const double dj = A.dist[min(r0 + (int)threadIdx.x, A.nr - 1)];
        ir_s[threadIdx.x] = (float)(1.0 / dj);
        ir_s[kN + threadIdx.x] = (float)(1.0 / (dj * dj));
    }
    if (warp == kMmaWarp) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tmem_base_s);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp == kCopyWarp) {
        // ---------------- bulk copies, up to SA stages ahead of the MMAs
        if (lane == 0) {
            const float *kt_tile = A.Kt + A.kt_base[wt];
            const float *braw = tiled ? A.B + (size_t)rt * A.bt_rows * NBASIS * kN : nullptr;
            int issued = 0;
            for (int st = 0; st < nstage; st++) {
                const int s = st % SA;
                if (st >= SA && !tc::mbar_wait_b(empty_bar(s), ((st / SA) - 1) & 1)) {
                    atomicOr(A.err, 2u);
                    fail_s = 1;
                    break;
                }
                if (fail_s) break;
                const int k0 = kb + st * KT;
                // this group's coefficient tiles of the (frequency tile, k stage) block
                // (a stage block is NQU x (hi, lo) tiles of 4 KB = 2048 floats per tile pair)
                const float *src = kt_tile + ((long long)(k0 / KT) * TG::NQU + TG::Q0) * (2 * kM * kKT);
                tc::mbar_expect_tx(land_bar(s), (uint32_t)TG::kABytes);
                tc::bulk_copy(sm_s + a_tile(s, 0, 0), src, (uint32_t)TG::kABytes, land_bar(s));
                if (tiled) {
                    tc::mbar_expect_tx(raw_bar(s), (uint32_t)TG::kRawBytes);
                    tc::bulk_copy(sm_s + raw_off(s), braw + (size_t)k0 * NBASIS * kN, (uint32_t)TG::kRawBytes,
                                  raw_bar(s));
                }
                issued = st + 1;
            }
            // copies still in flight are waited for (bounded) before the block may leave
            for (int st = max(0, issued - SA); st < issued; st++) {
                tc::mbar_wait_b(land_bar(st % SA), (st / SA) & 1);
                if (tiled) tc::mbar_wait_b(raw_bar(st % SA), (st / SA) & 1);
            }
        }
    } else if (warp < kProdWarps) {
        // ---------------- producers of the Bessel operand
        // (receiver, first k) of this thread in a stage: a warp covers one
        // 8-receiver x 32-byte core-matrix row block, so its B-operand stores
        // fill 32 distinct banks; KPT consecutive k per thread
        const int br = (warp & 3) * 8 + (lane >> 2), bk = (warp >> 2) * (4 * KPT) + (lane & 3) * KPT;
        const int rg = min(r0 + br, A.nr - 1);
        const bool rok = (r0 + br) < A.nr;
        const int ksm = A.ks ? A.ks[w0] : 1;
        const float dk = (float)(A.dk * ksm);
        // untiled table: Bessel values of the next stage loaded one stage ahead
        float bv[KPT][NBASIS];
        auto load_b = [&](int st_) {
#pragma unroll
            for (int i = 0; i < KPT; i++) {
                const int k = kb + st_ * KT + bk + i;
                const bool kok = st_ < nstage && k < ke && rok;
#pragma unroll
                for (int b = 0; b < NBASIS; b++)
                    if ((kBasis >> b) & 1u)
                        bv[i][b] = kok ? __ldg(A.B + ((long long)k * ksm * NBASIS + b) * A.nr + rg) : 0.f;
            }
        };
        if (!tiled) load_b(0);
        // each producer warp runs on its own (no barrier among them: the copy
        // thread refills a slot's raw rows only after its MMAs, which wait for
        // every producer's operand, hence after every producer has read them);
        // a wait that gives up in any lane ends the warp's loop (one decision
        // per warp, as its lanes share a __syncwarp)
        for (int st = 0; st < nstage; st++) {
            const int s = st % SA, sb = st % SB;
            const bool free_ok = st < SB || tc::mbar_wait_b(bempty_bar(sb), ((st / SB) - 1) & 1);
            if (__any_sync(0xffffffffu, !free_ok)) {
                atomicOr(A.err, 2u);
                fail_s = 1;
                break;
            }
            // B operand: pair values k^kp w J_b(k r) for (receiver br, k bk + i)
            float cur[KPT][NBASIS];
            if (tiled) {
                const bool raw_ok = tc::mbar_wait_b(raw_bar(s), (st / SA) & 1);
                if (__any_sync(0xffffffffu, !raw_ok)) {
                    atomicOr(A.err, 2u);
                    fail_s = 1;
                    break;
                }
                const float *rs = reinterpret_cast<const float *>(sm + raw_off(s));
#pragma unroll
                for (int i = 0; i < KPT; i++) {
                    // the tiled table permutes a row's receivers by r ^ 8 (k & 3); kb is a multiple of KT
                    const int kk = bk + i, bcol = br ^ ((kk & 3) << 3);
                    const bool kok = kb + st * KT + kk < ke && rok;
#pragma unroll
                    for (int b = 0; b < NBASIS; b++)
                        if ((kBasis >> b) & 1u) cur[i][b] = kok ? rs[(kk * NBASIS + b) * kN + bcol] : 0.f;
                }
            } else {
#pragma unroll
                for (int i = 0; i < KPT; i++)
#pragma unroll
                    for (int b = 0; b < NBASIS; b++) cur[i][b] = bv[i][b];
                load_b(st + 1);
            }
            float wk[KPT][3];
#pragma unroll
            for (int i = 0; i < KPT; i++) {
                const int k = kb + st * KT + bk + i;
                const float kf = dk * (float)k;
                const float w = (k == 0) ? 0.5f * dk : dk;
                wk[i][0] = w;
                wk[i][1] = w * kf;
                wk[i][2] = w * kf * kf;
            }
            const uint32_t boff = tc::tile_off<PREC>(br, bk);
#pragma unroll
            for (int slot = 0; slot < NP; slot++) {
                const Pair P = CT::pair(TP.gpair[GRP][slot]);
                if constexpr (PREC == kBF16) {
                    // two consecutive k of one receiver: their bf16 words share a 32-bit store
                    unsigned short h0, l0, h1, l1;
                    bf16_split(wk[0][P.kp] * cur[0][P.b], h0, l0);
                    bf16_split(wk[1][P.kp] * cur[1][P.b], h1, l1);
                    *reinterpret_cast<uint32_t *>(sm + b_tile(sb, slot, 0) + boff) = (uint32_t)h0 | ((uint32_t)h1 << 16);
                    *reinterpret_cast<uint32_t *>(sm + b_tile(sb, slot, 1) + boff) = (uint32_t)l0 | ((uint32_t)l1 << 16);
                } else {
                    const float v = wk[0][P.kp] * cur[0][P.b];
                    const float h = tc::tf32_rna(v), l = tc::tf32_rna(v - h);
                    *reinterpret_cast<float *>(sm + b_tile(sb, slot, 0) + boff) = h;
                    *reinterpret_cast<float *>(sm + b_tile(sb, slot, 1) + boff) = l;
                }
            }
            // make the generic-proxy writes visible to the tensor cores, then one
            // lane signals for the warp
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(full_bar(sb));
        }
    } else if (lane == 0) {
        // ---------------- MMA issuer (one thread of warp 9)
        for (int st = 0; st < nstage; st++) {
            const int s = st % SA, sb = st % SB;
            if (!tc::mbar_wait_b(land_bar(s), (st / SA) & 1) || !tc::mbar_wait_b(full_bar(sb), (st / SB) & 1)) {
                atomicOr(A.err, 4u);
                fail_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // fully unrolled: tile, operand and accumulator offsets are compile-time
            // constants; descriptors are the slots' base descriptors plus a constant
            // (b_tile(0, ...) carries the operand ring's offset after the copy ring)
            const uint64_t abase = tc::sdesc(sm_s + (uint32_t)(s * TG::kASlotBytes));
            const uint64_t bbase = tc::sdesc(sm_s + (uint32_t)(sb * TG::kBBytes));
            const uint32_t acc0 = st == 0 ? 0u : 1u;
            // the three split products of every column, round robin over the
            // columns: consecutive MMAs write different accumulators (the
            // order within one accumulator, hi*hi then hi*lo then lo*hi, stays)
#pragma unroll
            for (int sp3 = 0; sp3 < 3; sp3++)
#pragma unroll
                for (int i = 0; i < NQ; i++) {
                    const int first = TP.tfirst[TG::Q0 + i], count = TP.tcount[TG::Q0 + i];
                    const uint32_t idesc = tc::idesc_n<PREC>(count * kN);
                    const uint32_t d = tmem + (uint32_t)(first * kN);
                    const uint64_t a = abase + ((uint64_t)a_tile(0, i, sp3 == 2 ? 1 : 0) >> 4);
                    const uint64_t b = bbase + ((uint64_t)b_tile(0, first, sp3 == 1 ? 1 : 0) >> 4);
                    tc::mma_split<PREC>(d, a, b, idesc, sp3 == 0 ? acc0 : 1u);
                }
            // each commit arrives once every MMA issued so far is done: copy slot s
            // may then be refilled, operand slot sb rewritten
            tc::mma_commit(empty_bar(s));
            tc::mma_commit(bempty_bar(sb));
        }
        tc::mma_commit(done_bar);           // all MMAs of this CTA
    }

    // ---------------- drain: tensor memory -> partial sums
    if (warp < kProdWarps) {
        // the issuer always commits done_bar (immediately when it issued nothing)
        bool ok = nstage > 0;
        if (!tc::mbar_wait_b(done_bar, 0)) {
            atomicOr(A.err, 8u);
            ok = false;
        }
        if (fail_s) ok = false;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int quarter = warp & 3, half = warp >> 2;   // output columns c = half (mod 2)
        const int row = quarter * 32 + lane;              // the lane of tensor memory this thread reads
        const int part = row / kW, wl = row % kW, w = w0 + wl;
        const long long psplit = (long long)sp * 2 + GRP;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            if ((c & 1) != half) continue;
            float acc[kN];
#pragma unroll
            for (int j = 0; j < kN; j++) acc[j] = 0.f;
#pragma unroll
            for (int t = CT::col(c); t < CT::col(c + 1); t++) {
                const Term T = CT::term(t);
                if (TP.pgrp[T.pair] != GRP) continue;
                uint32_t v[kN];
                const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(TP.pslot[T.pair] * kN);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const float cf = (float)T.coef;
#pragma unroll
                for (int j = 0; j < kN; j++) {
                    const float f = T.rpow == 1 ? cf * ir_s[j] : T.rpow == 2 ? cf * ir_s[kN + j] : cf;
                    acc[j] = fmaf(f, __uint_as_float(v[j]), acc[j]);
                }
            }
            if (w < A.nw) {
#pragma unroll
                for (int j = 0; j < kN; j++) {
                    const int r = r0 + j;
                    if (r < A.nr) A.P[((((psplit * A.nr + r) * NC + c) * A.nw + w) * 2 + part)] = ok ? acc[j] : 0.f;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// Both column groups in one launch (even blocks group 0, odd blocks group 1),
// so that their CTAs share the waves of the SMs.  PREC: tc::kTF32 or tc::kBF16.
template <int SRC, int PREC>
__global__ void __launch_bounds__(tc::kThreads, 1) ksum_tc_kernel(KsumTcArgs<float> A)
{
    extern __shared__ __align__(1024) unsigned char smem_tc[];
    __shared__ __align__(8) unsigned long long bars[3 * tc::kMaxASlots + 2 * tc::kMaxBSlots + 1];   // copy ring, operand ring, done
    __shared__ float ir_s[2 * tc::kN];
    if (blockIdx.x & 1) ksum_tc_cta<SRC, 1, PREC>(A, (int)(blockIdx.x >> 1), smem_tc, bars, ir_s);
    else ksum_tc_cta<SRC, 0, PREC>(A, (int)(blockIdx.x >> 1), smem_tc, bars, ir_s);
}

// S[r][c][w] = sum over the partial sums (k slices x groups) with TwoSum
static __global__ void ksum_tc_reduce_kernel(const float *P, float *S, long long n, int nparts)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float hi = 0.f, lo = 0.f;
    for (int s = 0; s < nparts; s++) two_sum_acc(hi, lo, P[(long long)s * n + i]);
    S[i] = hi + lo;
}

}  // namespace grt
