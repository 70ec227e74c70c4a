// grt_ksum_tc.cuh -- the wavenumber integration on the tensor cores (tcgen05).
//
// For every output column c (get_int_val_single / _tensor, green.cu:1558-1716)
//   S_c(w, r) = sum_{t in c} coef_t r^-rpow_t D_{p(t)}(w, r),
//   D_p(w, r) = sum_k K_{q_p}(w, k) * w_k k^kp_p J_{b_p}(k r),
// one GEMM per pair p = (coefficient column q, power of k, Bessel function);
// the terms that share a pair differ only by a receiver-dependent factor,
// applied when the accumulators are drained.  The pairs are grouped by q, so
// that one MMA multiplies the coefficient tile of q by the Bessel operands of
// all its pairs at once (N = 16 receivers x pairs of q): each stage reads
// every coefficient tile from shared memory three times (3xTF32) instead of
// three times per term.  A CTA owns 64 frequencies (M = 128 rows: real parts
// in rows 0-63, imaginary parts in rows 64-127), 16 receivers and a slice of
// the k range (split-K); the accumulators of all pairs live in tensor memory
// (pairs x 16 columns).
//
// Precision: 3xTF32 -- each FP32 operand x is split into hi = tf32(x) and
// lo = tf32(x - hi) and the product is hi*hi + hi*lo + lo*hi with FP32
// accumulation (about 2^-21 relative per product).  Partial sums of the k
// slices are added with TwoSum by ksum_tc_reduce_kernel.
//
// Roles (160 threads): warps 0-3 produce operand tiles in shared memory
// (canonical K-major layout, no swizzle: 8-row x 16-byte core matrices) and
// drain the accumulators at the end; warp 4 allocates tensor memory and one
// of its threads issues tcgen05.mma and tcgen05.commit.  Two pipeline stages,
// each guarded by a "full" and an "empty" mbarrier.  Every wait is bounded:
// on timeout the CTA records an error, skips to the end, and still frees its
// tensor memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "grt_integrate.cuh"
#include "grt_types.h"

namespace grt {

namespace tc {

constexpr int kM = 128;        // rows: 64 frequencies x (re, im)
constexpr int kW = 64;         // frequencies per CTA
constexpr int kN = 16;         // receivers per CTA
constexpr int kKT = 8;         // k per stage = one tf32 MMA K
constexpr int kStages = 2;
constexpr int kProducers = 128;
constexpr int kThreads = kProducers + 32;
constexpr int kCoreBytes = 128;                      // 8 rows x 16 bytes
constexpr int kATileBytes = (kM / 8) * (kKT / 4) * kCoreBytes;   // 4096: one q, one split
constexpr int kBTileBytes = (kN / 8) * (kKT / 4) * kCoreBytes;   // 512: one term, one split
constexpr uint32_t kTmemCols = 512;

template <int SRC> struct TcCfg {
    static constexpr int NQ = Cols<SRC>::NQ, NC = Cols<SRC>::NC, NP = Cols<SRC>::NP;
};

// the pairs in order of their coefficient column q: slot[p] is pair p's
// position, first[q] / count[q] the run of q's pairs
template <int SRC> struct PairGroups {
    int order[32], slot[32], first[16], count[16];
};
template <int SRC> constexpr PairGroups<SRC> make_groups()
{
    PairGroups<SRC> g{};
    int n = 0;
    for (int q = 0; q < Cols<SRC>::NQ; q++) {
        g.first[q] = n;
        g.count[q] = 0;
        for (int p = 0; p < Cols<SRC>::NP; p++)
            if (Cols<SRC>::pair(p).q == q) {
                g.order[n] = p;
                g.slot[p] = n;
                n++;
                g.count[q]++;
            }
    }
    return g;
}

template <int SRC> constexpr int stage_bytes()
{
    return TcCfg<SRC>::NQ * 2 * kATileBytes + TcCfg<SRC>::NP * 2 * kBTileBytes;
}
// raw Bessel rows of one stage: 8 rows x NBASIS x 16 receivers (tiled table)
constexpr int kRawBytes = kKT * NBASIS * kN * 4;
template <int SRC> constexpr int smem_bytes() { return kStages * (stage_bytes<SRC>() + kRawBytes) + 1024; }

static_assert(kKT == kTileK && kM == kTileRows, "tile shape shared with the GRT kernel");
__device__ __forceinline__ uint32_t tile_off(int row, int k) { return kt_tile_off(row, k); }

// shared-memory matrix descriptor: K-major, no swizzle.  LBO = distance of
// core matrices adjacent in K (128 B), SBO = distance of 8-row groups.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    const uint64_t lbo = kCoreBytes, sbo = (uint64_t)(kKT / 4) * kCoreBytes;
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(lbo >> 4) << 16;
    d |= (uint64_t)(sbo >> 4) << 32;
    d |= (uint64_t)1 << 46;       // descriptor version for sm_100-family tensor cores
    return d;                     // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor: dense, D = F32, A = B = TF32, both K-major, M = 128, N = n
constexpr uint32_t idesc_n(int n)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
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
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

}  // namespace tc

template <typename R>
struct KsumTcArgs {
    const float *Kt;         // operand blocks written by the GRT kernel (see GrtArgs::Kt)
    const long long *kt_base;
    const float *B;          // [nbrow][NBASIS][nr], row i at k = i dk; or tiled (bt_rows > 0)
    int bt_rows;             // > 0: B is [nr / 16][bt_rows][NBASIS][16] (unit strides only)
    const int *nk;           // [nw]
    const int *ks;           // [nw] k stride, constant on each tile of kW frequencies (null: 1)
    const long long *koff;   // [nw]
    const double *dist;      // [nr]
    float *P;                // partial sums [nsplit][nr][nc][nw] complex
    long long nkw;
    double dk;
    int nw, nr, nkmax, nsplit, kslice;   // kslice: k per split (multiple of kKT)
    unsigned int *err;
};

template <int SRC>
__global__ void __launch_bounds__(tc::kThreads, 1) ksum_tc_kernel(KsumTcArgs<float> A)
{
    using namespace tc;
    using CT = Cols<SRC>;
    constexpr int NQ = TcCfg<SRC>::NQ, NC = TcCfg<SRC>::NC, NP = TcCfg<SRC>::NP;
    constexpr PairGroups<SRC> G = make_groups<SRC>();
    static_assert(NP * kN <= (int)kTmemCols, "accumulators exceed tensor memory");
    extern __shared__ __align__(1024) unsigned char smem_tc[];
    __shared__ __align__(8) unsigned long long bars[3 * kStages + 1];
    __shared__ uint32_t tmem_base_s;
    __shared__ int fail_s;

    const int nrt = (A.nr + kN - 1) / kN;
    const int wt = blockIdx.x / (nrt * A.nsplit);
    const int rem = blockIdx.x % (nrt * A.nsplit);
    const int rt = rem / A.nsplit, sp = rem % A.nsplit;
    const int w0 = wt * kW, r0 = rt * kN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // k range of this CTA: [kb, ke) within the longest frequency of the tile
    int nkt = 0;
    for (int i = 0; i < kW; i++)
        if (w0 + i < A.nw) nkt = max(nkt, A.nk[w0 + i]);
    const int kb = sp * A.kslice;
    const int ke = min(nkt, kb + A.kslice);
    const int nstage = ke > kb ? (ke - kb + kKT - 1) / kKT : 0;

    unsigned char *sm = (unsigned char *)(((uintptr_t)smem_tc + 1023) & ~(uintptr_t)1023);
    const uint32_t sm_s = (uint32_t)__cvta_generic_to_shared(sm);
    auto full_bar = [&](int s) { return (uint32_t)__cvta_generic_to_shared(&bars[s]); };
    auto empty_bar = [&](int s) { return (uint32_t)__cvta_generic_to_shared(&bars[kStages + s]); };
    const uint32_t done_bar = (uint32_t)__cvta_generic_to_shared(&bars[2 * kStages]);
    auto raw_bar = [&](int s) { return (uint32_t)__cvta_generic_to_shared(&bars[2 * kStages + 1 + s]); };
    const bool tiled = A.bt_rows > 0;
    auto raw_off = [&](int s) { return (uint32_t)(kStages * stage_bytes<SRC>() + s * kRawBytes); };
    auto a_tile = [&](int s, int q, int split) {
        return (uint32_t)(s * stage_bytes<SRC>() + (q * 2 + split) * kATileBytes);
    };
    // B operands: split-major, pairs in q order, 16 rows (receivers) per pair
    auto b_tile = [&](int s, int slot, int split) {
        return (uint32_t)(s * stage_bytes<SRC>() + NQ * 2 * kATileBytes + (split * NP + slot) * kBTileBytes);
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            // every producer arrives once, plus producer 0's expect-tx arrival for the A copy
            tc::mbar_init(full_bar(s), kProducers + 1);
            tc::mbar_init(empty_bar(s), 1);
        }
        tc::mbar_init(done_bar, 1);
        for (int s = 0; s < kStages; s++) tc::mbar_init(raw_bar(s), 1);
        fail_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tmem_base_s);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp < 4) {
        // ---------------- producers
        const int tid = threadIdx.x;
        // (receiver, k) of this thread in a stage: a warp covers one 8-receiver x
        // 4-k core matrix, so its B-operand stores fill 32 distinct banks
        const int br = (warp & 1) * 8 + (lane >> 2), bk = (warp >> 1) * 4 + (lane & 3);
        const int rg = min(r0 + br, A.nr - 1);
        const bool rok = (r0 + br) < A.nr;
        const int ksm = A.ks ? A.ks[w0] : 1;
        const float dk = (float)(A.dk * ksm);
        const unsigned a_bytes = (unsigned)(NQ * 2 * kATileBytes);
        const float *kt_tile = A.Kt + A.kt_base[wt];
        const float *braw = tiled ? A.B + (size_t)rt * A.bt_rows * NBASIS * kN : nullptr;
        // tiled table: the raw rows of a stage arrive by one bulk copy, a stage ahead
        auto issue_raw = [&](int st_) {
            const int s_ = st_ % kStages;
            const float *src = braw + (size_t)(kb + st_ * kKT) * NBASIS * kN;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(raw_bar(s_)),
                         "r"((unsigned)kRawBytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    sm_s + raw_off(s_)),
                "l"(src), "r"((unsigned)kRawBytes), "r"(raw_bar(s_))
                : "memory");
        };
        int raw_issued = 0;
        if (tiled && tid == 0 && nstage > 0) {
            issue_raw(0);
            raw_issued = 1;
        }
        // untiled table: Bessel values of the next stage loaded one stage ahead
        float bv[NBASIS];
        auto load_b = [&](int st_) {
            const int k = kb + st_ * kKT + bk;
            const bool kok = st_ < nstage && k < ke && rok;
#pragma unroll
            for (int b = 0; b < NBASIS; b++) bv[b] = kok ? __ldg(A.B + ((long long)k * ksm * NBASIS + b) * A.nr + rg) : 0.f;
        };
        if (!tiled) load_b(0);
        for (int st = 0; st < nstage; st++) {
            const int s = st % kStages;
            if (st >= kStages) {
                if (!tc::mbar_wait_b(empty_bar(s), ((st / kStages) - 1) & 1)) {
                    atomicOr(A.err, 2u);
                    fail_s = 1;
                }
            }
            // all producers are past stage st - 1 (its raw buffer may be refilled) and
            // take one decision on failure: the OR over the producers of what each saw
            // (the issuing warp may set fail_s at any time)
            int any_fail;
            asm volatile(
                "{\n\t.reg .pred p, q;\n\t"
                "setp.ne.s32 p, %1, 0;\n\t"
                "bar.red.or.pred q, 1, %2, p;\n\t"
                "selp.s32 %0, 1, 0, q;\n\t}\n"
                : "=r"(any_fail)
                : "r"((int)fail_s), "n"(kProducers)
                : "memory");
            if (any_fail) break;
            const int k0 = kb + st * kKT;
            if (tid == 0) {
                if (tiled && st + 1 < nstage) {
                    issue_raw(st + 1);
                    raw_issued = st + 2;
                }
                // A operand: one bulk copy of the (frequency tile, k stage) block the
                // GRT kernel wrote in operand layout
                const float *src = kt_tile + (long long)(k0 / kKT) * (NQ * 2 * kM * kKT);
                const uint32_t dst = sm_s + a_tile(s, 0, 0);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full_bar(s)), "r"(a_bytes)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                    "l"(src), "r"(a_bytes), "r"(full_bar(s))
                    : "memory");
            }
            // B operand: pair values k^kp w J_b(k r) for (receiver br, k bk)
            {
                const int k = k0 + bk;
                float cur[NBASIS];
                if (tiled) {
                    if (!tc::mbar_wait_b(raw_bar(s), (st / kStages) & 1)) {
                        atomicOr(A.err, 2u);
                        fail_s = 1;
                    }
                    const float *rs = reinterpret_cast<const float *>(sm + raw_off(s));
                    const bool kok = k < ke && rok;
#pragma unroll
                    for (int b = 0; b < NBASIS; b++) cur[b] = kok ? rs[(bk * NBASIS + b) * kN + br] : 0.f;
                } else {
#pragma unroll
                    for (int b = 0; b < NBASIS; b++) cur[b] = bv[b];
                    load_b(st + 1);
                }
                const float kf = dk * (float)k;
                const float w = (k == 0) ? 0.5f * dk : dk;
                const float wk[3] = {w, w * kf, w * kf * kf};
#pragma unroll
                for (int p = 0; p < NP; p++) {
                    const Pair P = CT::pair(p);
                    const float v = wk[P.kp] * cur[P.b];
                    const float h = tc::tf32_rna(v), l = tc::tf32_rna(v - h);
                    *reinterpret_cast<float *>(sm + b_tile(s, G.slot[p], 0) + tc::tile_off(br, bk)) = h;
                    *reinterpret_cast<float *>(sm + b_tile(s, G.slot[p], 1) + tc::tile_off(br, bk)) = l;
                }
            }
            // make the generic-proxy writes visible to the tensor cores, then signal
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc::mbar_arrive(full_bar(s));
        }
        // a raw copy issued for a stage that was never consumed (early exit) is
        // waited for (bounded) before the block can leave
        if (tiled && tid == 0 && raw_issued > 0) {
            const int last = raw_issued - 1;
            tc::mbar_wait_b(raw_bar(last % kStages), (last / kStages) & 1);
        }
    } else if (lane == 0) {
        // ---------------- MMA issuer (one thread of warp 4)
        for (int st = 0; st < nstage; st++) {
            const int s = st % kStages;
            if (!tc::mbar_wait_b(full_bar(s), (st / kStages) & 1)) {
                atomicOr(A.err, 4u);
                fail_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // fully unrolled: group, operand and accumulator offsets are compile-time
            // constants; descriptors are the stage's base descriptor plus a constant
            const uint64_t dbase = tc::sdesc(sm_s + (uint32_t)(s * stage_bytes<SRC>()));
            const uint32_t acc0 = st == 0 ? 0u : 1u;
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                if (G.count[q] == 0) continue;
                const uint32_t idesc = tc::idesc_n(G.count[q] * kN);
                const uint32_t d = tmem + (uint32_t)(G.first[q] * kN);
                const uint64_t ah = dbase + ((uint64_t)a_tile(0, q, 0) >> 4), al = dbase + ((uint64_t)a_tile(0, q, 1) >> 4);
                const uint64_t bh = dbase + ((uint64_t)b_tile(0, G.first[q], 0) >> 4);
                const uint64_t bl = dbase + ((uint64_t)b_tile(0, G.first[q], 1) >> 4);
                tc::mma_tf32(d, ah, bh, idesc, acc0);
                tc::mma_tf32(d, ah, bl, idesc, 1u);
                tc::mma_tf32(d, al, bh, idesc, 1u);
            }
            tc::mma_commit(empty_bar(s));   // stage s may be refilled once these MMAs finish
        }
        tc::mma_commit(done_bar);           // all MMAs of this CTA
    }

    // ---------------- drain: tensor memory -> partial sums
    if (warp < 4) {
        // the issuer always commits done_bar (immediately when it issued nothing)
        bool ok = nstage > 0;
        if (!tc::mbar_wait_b(done_bar, 0)) {
            atomicOr(A.err, 8u);
            ok = false;
        }
        if (fail_s) ok = false;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int row = warp * 32 + lane;            // the lane of tensor memory this thread reads
        const int part = row / kW, wl = row % kW, w = w0 + wl;
        // receiver factors r^-1, r^-2 of the terms
        float irj[kN], ir2j[kN];
#pragma unroll
        for (int j = 0; j < kN; j++) {
            const double dj = A.dist[min(r0 + j, A.nr - 1)];
            irj[j] = (float)(1.0 / dj);
            ir2j[j] = (float)(1.0 / (dj * dj));
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            float acc[kN];
#pragma unroll
            for (int j = 0; j < kN; j++) acc[j] = 0.f;
#pragma unroll
            for (int t = CT::col(c); t < CT::col(c + 1); t++) {
                const Term T = CT::term(t);
                uint32_t v[kN];
                const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(G.slot[T.pair] * kN);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(taddr)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const float cf = (float)T.coef;
#pragma unroll
                for (int j = 0; j < kN; j++) {
                    const float f = T.rpow == 1 ? cf * irj[j] : T.rpow == 2 ? cf * ir2j[j] : cf;
                    acc[j] = fmaf(f, __uint_as_float(v[j]), acc[j]);
                }
            }
            if (w < A.nw) {
#pragma unroll
                for (int j = 0; j < kN; j++) {
                    const int r = r0 + j;
                    if (r < A.nr) A.P[((((long long)sp * A.nr + r) * NC + c) * A.nw + w) * 2 + part] = ok ? acc[j] : 0.f;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 4) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// S[r][c][w] = sum over k slices of the partial sums (TwoSum)
__global__ void ksum_tc_reduce_kernel(const float *P, float *S, long long n, int nsplit)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float hi = 0.f, lo = 0.f;
    for (int s = 0; s < nsplit; s++) two_sum_acc(hi, lo, P[(long long)s * n + i]);
    S[i] = hi + lo;
}

}  // namespace grt
