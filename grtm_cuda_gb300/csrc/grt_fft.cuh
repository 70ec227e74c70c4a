// grt_fft.cuh -- the FP32 spectral stage as a bandwidth kernel: per trace,
// phase/taper/scale, Hermitian fill, inverse DFT and de-damping
// (green.cu:1905-1938, 2222-2239), without materialising the filled
// spectrum.
//
// The reference fills out[0..N) Hermitian (out[N-n] = conj(out[n]),
// out[nw] = 0), runs a complex inverse FFT of length N and keeps the real
// part.  Keeping the real part is the same as transforming the Hermitian
// sequence with out[0] replaced by Re out[0], and the inverse transform of a
// Hermitian sequence of length N = 2M is one complex transform of length M:
//
//   Z[k] = (X[k] + conj X[M-k]) + i e^{2 pi i k/N} (X[k] - conj X[M-k])
//   z = IDFT_M(Z),  x[2n] = Re z[n],  x[2n+1] = Im z[n]
//
// (X[k] = S[k] post[k], k < M; Z[0] = Re X[0] (1 + i) since X[M] = 0).  The
// length-M transform is a Stockham radix-16 FFT: E = 16 values per thread
// (fewer for M < 16), M/E threads per trace, radix-16 passes and one final
// radix-2/4/8 pass when log2 M is not a multiple of 4.  The first pass takes
// its inputs straight from global memory, the last writes the de-damped
// samples straight to global memory (coalesced float2 stores); the passes in
// between exchange through one padded shared-memory buffer (index
// a + a/16: conflict-free for the stride-16 writes of the first pass and the
// unit-stride reads and writes of the others).  The twiddles of pass p > 0,
// e^{2 pi i r s / (Ns R)} (r = 1..R-1, s = b mod Ns), come from a table laid
// out [pass][r - 1][s]: a warp's lanes read consecutive s, one or two L1
// wavefronts per load (indexing one e^{2 pi i m/N} table by r s scatters the
// lanes over up to 32 lines, and the load pipe, not DRAM, limited the
// kernel).  The table has M - 16 entries: (R - 1) Ns summed over the passes
// telescopes to M - Ns of the second pass.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

namespace grt {
namespace fft {

// cos and sin of pi/8, sqrt(1/2)
constexpr float kC8 = 0.923879532511286756f;
constexpr float kS8 = 0.382683432365089772f;
constexpr float kR2 = 0.707106781186547524f;

__device__ __forceinline__ float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 mul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// v e^{2 pi i q / 16}, q = 0..7 (a constant once the transform is unrolled)
__device__ __forceinline__ float2 rot16(float2 v, int q)
{
    switch (q) {
    case 0: return v;
    case 1: return make_float2(kC8 * v.x - kS8 * v.y, kS8 * v.x + kC8 * v.y);
    case 2: return make_float2(kR2 * (v.x - v.y), kR2 * (v.x + v.y));
    case 3: return make_float2(kS8 * v.x - kC8 * v.y, kC8 * v.x + kS8 * v.y);
    case 4: return make_float2(-v.y, v.x);
    case 5: return make_float2(-kS8 * v.x - kC8 * v.y, kC8 * v.x - kS8 * v.y);
    case 6: return make_float2(-kR2 * (v.x + v.y), kR2 * (v.x - v.y));
    default: return make_float2(-kC8 * v.x - kS8 * v.y, kS8 * v.x - kC8 * v.y);
    }
}

// in-register inverse DFT of length R (2, 4, 8, 16), natural order in and
// out: y[k] = sum_n v[n] e^{+2 pi i nk/R}; radix-2 decimation in time on the
// bit-reversed registers
template <int R>
__device__ __forceinline__ void dft(float2 *v)
{
    constexpr int LR = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
#pragma unroll
    for (int i = 0; i < R; i++) {
        int ri = 0;
#pragma unroll
        for (int b = 0; b < LR; b++) ri |= ((i >> b) & 1) << (LR - 1 - b);
        if (i < ri) {
            const float2 t = v[i];
            v[i] = v[ri];
            v[ri] = t;
        }
    }
#pragma unroll
    for (int half = 1; half < R; half *= 2)
#pragma unroll
        for (int g = 0; g < R; g += 2 * half)
#pragma unroll
            for (int pos = 0; pos < half; pos++) {
                const float2 u = v[g + pos], w = rot16(v[g + pos + half], pos * 8 / half);
                v[g + pos] = add(u, w);
                v[g + pos + half] = sub(u, w);
            }
}

__device__ __forceinline__ int pad(int a) { return a + (a >> 4); }

template <int LOGM>
struct Shape {
    static constexpr int M = 1 << LOGM;
    static constexpr int E = M < 16 ? M : 16;      // values per thread
    static constexpr int T = M / E;                // threads per trace
    static constexpr int NP = (LOGM + 3) / 4;      // passes
    static constexpr int smem_bytes = NP > 1 ? (M + M / 16) * 8 : 0;
    static constexpr int radix(int p) { return p < LOGM / 4 ? 16 : 1 << (LOGM % 4); }
    static constexpr int span(int p) { return p == 0 ? 1 : 16 * span(p - 1); }   // Ns: product of earlier radices
};

struct C2RArgs {
    const float2 *S;       // [ntr][M] wavenumber sums
    const float2 *post;    // [M] phase, taper, scale
    const float2 *tw;      // [M] e^{2 pi i m / N}
    const float2 *twp;     // [M - 16] the passes' twiddles (pass_twiddles)
    const float *damp;     // [N] e^{sigma (n dt + t0)} / N
    float *out;            // [ntr][N]
};

// entries of the pass twiddle table of a length-2^logm transform
__host__ __device__ constexpr int pass_twiddle_count(int logm) { return logm > 4 ? (1 << logm) - 16 : 0; }

// the pass twiddle table of N = 2^logn (2 <= logn <= 15) as interleaved
// (re, im) floats: for each pass p >= 1 (radix R, span Ns), for r = 1..R-1,
// for s = 0..Ns-1, e^{2 pi i r s / (Ns R)}, rounded from double
static inline void pass_twiddles(int logn, float *out)
{
    const int logm = logn - 1, np = (logm + 3) / 4;
    long long o = 0;
    int ns = 16;
    for (int p = 1; p < np; p++) {
        const int R = p < logm / 4 ? 16 : 1 << (logm % 4);
        for (int r = 1; r < R; r++)
            for (int s = 0; s < ns; s++) {
                const double a = 2.0 * 3.14159265358979323846 * r * s / ((double)ns * R);
                out[2 * o] = (float)std::cos(a);
                out[2 * o + 1] = (float)std::sin(a);
                o++;
            }
        ns *= R;
    }
}

// pass P of the length-M transform on v (E values of this thread); P > 0
// first gathers its inputs from the shared buffer and applies the twiddles
template <int LOGM, int P>
struct Pass {
    static __device__ __forceinline__ void run(float2 (&v)[16], float2 *sm, int j, const float2 *__restrict__ twp,
                                               const float2 *__restrict__ damp2, float2 *__restrict__ out)
    {
        using Sh = Shape<LOGM>;
        constexpr int M = Sh::M, T = Sh::T, E = Sh::E;
        constexpr int R = Sh::radix(P), Ns = Sh::span(P), H = E / R;
        if constexpr (P > 0) {
#pragma unroll
            for (int h = 0; h < H; h++)
#pragma unroll
                for (int r = 0; r < R; r++) v[h * R + r] = sm[pad(j + h * T + r * (M / R))];
            if constexpr (P < Sh::NP - 1) __syncthreads();   // every read done before this pass writes
            // this pass's block of the table starts after the earlier passes' (R - 1) Ns entries
            const float2 *__restrict__ tp = twp + (Ns - 16);
#pragma unroll
            for (int h = 0; h < H; h++) {
                const int s = (j + h * T) % Ns;
#pragma unroll
                for (int r = 1; r < R; r++) v[h * R + r] = mul(v[h * R + r], __ldg(tp + (r - 1) * Ns + s));
            }
        }
#pragma unroll
        for (int h = 0; h < H; h++) dft<R>(v + h * R);
        if constexpr (P == Sh::NP - 1) {
            // b < M/R: the output index of (b, r) is b + r M/R; z[n] -> x[2n], x[2n+1]
#pragma unroll
            for (int h = 0; h < H; h++)
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int n = j + h * T + r * (M / R);
                    const float2 d = __ldg(damp2 + n);
                    out[n] = make_float2(v[h * R + r].x * d.x, v[h * R + r].y * d.y);
                }
        } else {
#pragma unroll
            for (int h = 0; h < H; h++) {
                const int b = j + h * T;
                const int e = (b / Ns) * Ns * R + b % Ns;
#pragma unroll
                for (int r = 0; r < R; r++) sm[pad(e + r * Ns)] = v[h * R + r];
            }
            __syncthreads();
            Pass<LOGM, P + 1>::run(v, sm, j, twp, damp2, out);
        }
    }
};

// one CTA of M/E threads per trace
template <int LOGM>
__global__ void __launch_bounds__(Shape<LOGM>::T) c2r_kernel(C2RArgs A)
{
    using Sh = Shape<LOGM>;
    constexpr int M = Sh::M, T = Sh::T, E = Sh::E;
    extern __shared__ float2 smem_c2r[];
    const int j = threadIdx.x;
    const long long tr = blockIdx.x;
    const float2 *__restrict__ S = A.S + tr * M;
    const float2 *__restrict__ post = A.post;
    float2 v[16];
    // Z[k], k = j + r T: the first pass's inputs
#pragma unroll
    for (int r = 0; r < E; r++) {
        const int k = j + r * T;
        const float2 x = mul(__ldg(S + k), __ldg(post + k));
        if (k == 0) {
            v[r] = make_float2(x.x, x.x);
        } else {
            const float2 y = mul(__ldg(S + (M - k)), __ldg(post + (M - k)));
            const float2 a = make_float2(x.x + y.x, x.y - y.y);
            const float2 b = mul(make_float2(x.x - y.x, x.y + y.y), __ldg(A.tw + k));
            v[r] = make_float2(a.x - b.y, a.y + b.x);
        }
    }
    Pass<LOGM, 0>::run(v, smem_c2r, j, A.twp, reinterpret_cast<const float2 *>(A.damp),
                       reinterpret_cast<float2 *>(A.out) + tr * M);
}

template <int LOGM>
static cudaError_t launch_c2r_m(const C2RArgs &A, long long ntr, cudaStream_t st)
{
    using Sh = Shape<LOGM>;
    if (Sh::smem_bytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(c2r_kernel<LOGM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             Sh::smem_bytes);
        if (e != cudaSuccess) return e;
    }
    c2r_kernel<LOGM><<<(unsigned)ntr, Sh::T, Sh::smem_bytes, st>>>(A);
    return cudaGetLastError();
}

// set the kernels' shared-memory limits outside a stream capture
static inline cudaError_t c2r_prepare(int logn)
{
    switch (logn - 1) {
    case 13: return cudaFuncSetAttribute(c2r_kernel<13>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Shape<13>::smem_bytes);
    case 14: return cudaFuncSetAttribute(c2r_kernel<14>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Shape<14>::smem_bytes);
    default: return cudaSuccess;
    }
}

// the spectral stage of ntr traces of length N = 2^logn (2 <= logn <= 15)
static inline cudaError_t launch_c2r(const C2RArgs &A, long long ntr, int logn, cudaStream_t st)
{
    if (ntr <= 0) return cudaSuccess;
    switch (logn - 1) {
    case 1: return launch_c2r_m<1>(A, ntr, st);
    case 2: return launch_c2r_m<2>(A, ntr, st);
    case 3: return launch_c2r_m<3>(A, ntr, st);
    case 4: return launch_c2r_m<4>(A, ntr, st);
    case 5: return launch_c2r_m<5>(A, ntr, st);
    case 6: return launch_c2r_m<6>(A, ntr, st);
    case 7: return launch_c2r_m<7>(A, ntr, st);
    case 8: return launch_c2r_m<8>(A, ntr, st);
    case 9: return launch_c2r_m<9>(A, ntr, st);
    case 10: return launch_c2r_m<10>(A, ntr, st);
    case 11: return launch_c2r_m<11>(A, ntr, st);
    case 12: return launch_c2r_m<12>(A, ntr, st);
    case 13: return launch_c2r_m<13>(A, ntr, st);
    case 14: return launch_c2r_m<14>(A, ntr, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace fft
}  // namespace grt
