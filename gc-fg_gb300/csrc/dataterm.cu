// dataterm.cu -- colour-histogram t-links, contrast-sensitive n-links and
// the fused image -> tile-space residual graph build, for a whole batch.
//
// Replaces the reference's data-term module (DataTerm.cpp:52-205,
// DataTermKernels.cu:19-150), whose Gaussian KDE over a 256^3 cube is
// replaced by a 16^3 colour histogram per class:
//   p_k(bin) = (H_k[bin] + 1) / (N_k + 4096),  bin = (r>>4, g>>4, b>>4)
//   dp = round(10 * -log p_bg)   (source / foreground t-link)
//   dn = round(10 * -log p_fg)   (sink / background t-link)
// N-links: w = round(lambda * exp(-||dI||^2 / (2 sigma^2))), sigma^2 = mean
// ||dI||^2 over all horizontally and vertically adjacent pairs.  The
// reference has no n-link kernel; its callers pass per-direction arrays
// (solveMRF.cu:87-90) that InitGraphVarEdges consumes
// (GraphCutKernels.cu:165-214).
//
// Exactness: the CPU oracle evaluates these expressions in double precision.
// Here the 4096 per-bin t-links of an image go into a table, and the n-link
// of every pixel pair is evaluated directly; both use a float evaluation
// whenever it is provably far from a rounding boundary and the oracle's
// double expression otherwise, so every int32 capacity matches bit for bit.
#include <cstring>

#include "dataterm.cuh"

namespace gcfg {

__device__ __forceinline__ int color_bin3(const uint8_t *__restrict__ p) {
    return ((p[0] >> 4) << 8) | ((p[1] >> 4) << 4) | (p[2] >> 4);
}

__device__ __forceinline__ int diff2p(const uint8_t *__restrict__ a, const uint8_t *__restrict__ b) {
    const int d0 = (int)a[0] - b[0], d1 = (int)a[1] - b[1], d2 = (int)a[2] - b[2];
    return d0 * d0 + d1 * d1 + d2 * d2;
}

// Colour of a pixel as one word: r | g << 8 | b << 16.
__device__ __forceinline__ uint32_t pack_rgb(const uint8_t *__restrict__ p) {
    return (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8) | ((uint32_t)__ldg(p + 2) << 16);
}

// ||a - b||^2 of two packed colours: per-byte absolute differences, then the
// dot product of that word with itself (the top byte is 0 in both).
__device__ __forceinline__ int diff2w(uint32_t a, uint32_t b) {
    const uint32_t d = __vabsdiffu4(a, b);
    return (int)__dp4a(d, d, 0u);
}

__device__ __forceinline__ int color_binw(uint32_t c) {
    return (((c >> 4) & 0xFu) << 8) | (((c >> 12) & 0xFu) << 4) | ((c >> 20) & 0xFu);
}

// ---------------------------------------------------------------------------
// Quantised table entries.  The reference value is the double expression
// the CPU oracle evaluates; a float evaluation decides the rounding whenever
// it lies farther from a .5 boundary than its proven error, and the double
// expression is evaluated only for the near-ties that remain.
// ---------------------------------------------------------------------------

// 10 * -ln((h + 1) / N) in double (the oracle's expression).  Not inlined,
// so that the compiler cannot speculate it into the float fast path.
__device__ __noinline__ double tlink_raw(int h, long long N) {
    const double p = (double)(h + 1) / (double)N;
    return 10.0 * -log(p);
}

// round(10 * -ln((h+1)/N)).  Float error: the ratio carries <= 3 ulp
// (conversions and division, 1.8e-7 relative), which moves the log by
// <= 1.8e-7; logf adds <= 1 ulp of a result <= 22 (2.7e-6); times 10:
// < 3e-5.  Margin used: 1e-3.
__device__ __forceinline__ int tlink_quant(int h, long long N) {
    const float pf = (float)(h + 1) / (float)N;
    const float v = -10.0f * logf(pf);
    const float fr = v - floorf(v);
    if (fabsf(fr - 0.5f) > 1e-3f) return (int)floorf(v + 0.5f);
    return (int)round(tlink_raw(h, N));
}

// round(lambda * exp(-d2 / (2 s2))).  The fast path evaluates
// v = lf * 2^z, z = -d2 * scale, scale = (float)(log2(e) / (2 s2)), with one
// ex2.approx.ftz.f32 (the hardware base-2 exponential; PTX documents a
// maximum relative error of about 2^-22, and gcfg_selftest_ex2 measures it
// over [-64, 0] on the device, where the tests require <= 2^-21).  Error of
// v: d2 is exact; scale and the product round once each, so z is off by
// <= 2^-23 |z|, i.e. 2^z by a relative 1.2e-7 |a| with a = z ln 2 the
// natural exponent; ex2 adds <= 2^-21 (4.8e-7); lf = (float)lambda and the
// final product <= 0.5 ulp each (1.2e-7): v is off by < v * (1.2e-7 |a| +
// 7.2e-7).  A wrong rounding needs v within that error of some k + 0.5,
// where v <= lambda and |a| = ln(lambda / (k + 0.5)) <= ln(2 lambda): the
// error is then < lambda * (1.2e-7 ln(2 lambda) + 7.2e-7).  The margin used
// is about twice that: lambda * (2.5e-7 ln(2 lambda + 1) + 1.5e-6) + 1e-6,
// set per image.  Within the margin the double expression decides.  (Large
// |a| only make v smaller: it underflows toward 0 and rounds to 0.)
//
// The fast path uses no conversion instructions (they share a slow pipe on
// this GPU): d2 < 2^23 becomes a float by writing it into the mantissa of
// 2^23, and for lambda < 2^22 the nearest integer of v comes from adding
// 1.5 * 2^23 (round to nearest even; exact ties cannot pass the margin test).
// v is at distance 0.5 - |v - rint(v)| from the nearest k + 0.5, so the
// margin test reads |v - rint(v)| < 0.5 - margin.
struct NlinkParams {
    float lf, scale;     // (float)lambda, (float)(log2(e) / (2 sigma^2))
    float margin;        // per image, from the error bound above
    float half_margin;   // 0.5 - margin
    int small;           // lambda < 2^22: the magic-number rounding applies
    int constant;        // constant image: every weight is const_w = round(lambda)
    int const_w;
    double lambda, s2;   // only read on the exact (near-tie) path
};

// round(lambda * exp(-d2 / (2 s2))) in double: the oracle's expression.  Not
// inlined, so that it cannot be speculated into the float fast path.
__device__ __noinline__ int nlink_exact(int d2, double lambda, double s2) {
    const double a = -(double)d2 / (2.0 * s2);
    return (int)round(lambda * exp(a));
}

// sigma^2 and 1 / (2 sigma^2) of each image, once per image.
__global__ void k_img_params(const int *__restrict__ ilist, const ImgDesc *__restrict__ img, int n_img,
                             ImgState *ist) {
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_img) return;
    const int im = ilist ? ilist[li] : li;
    const unsigned long long s = ist[im].sigma_sum;
    const long long count = (long long)(img[im].W - 1) * img[im].H + (long long)img[im].W * (img[im].H - 1);
    const double s2 = (s == 0 || count == 0) ? 0.0 : (double)s / (double)count;
    ist[im].s2 = s2;
    ist[im].ex2_scale = s2 > 0.0 ? (float)(1.4426950408889634 / (2.0 * s2)) : 0.f;  // log2(e) / (2 s2)
    ist[im].lambda_f = (float)img[im].lambda;
    ist[im].const_w = (int)round(img[im].lambda);
    const double lam = img[im].lambda;
    ist[im].nl_margin = (float)(lam * (2.5e-7 * log(2.0 * lam + 1.0) + 1.5e-6) + 1e-6);
}

__device__ __forceinline__ NlinkParams nlink_params(double lambda, const ImgState &st) {
    NlinkParams q;
    q.lambda = lambda;
    q.s2 = st.s2;
    q.lf = st.lambda_f;
    q.scale = st.ex2_scale;
    q.constant = st.ex2_scale == 0.f;
    q.const_w = st.const_w;
    q.margin = st.nl_margin;
    q.half_margin = 0.5f - q.margin;
    q.small = q.lf < 4194304.0f;
    return q;
}

// Exact float of 0 <= d2 < 2^23 (squared colour distances are <= 3 * 255^2).
__device__ __forceinline__ float small_int_to_float(int d2) {
    return __fsub_rn(__int_as_float(0x4B000000 | d2), 8388608.0f);
}

__device__ __forceinline__ float ex2_approx(float z) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(z));
    return r;
}

// The float fast path: w = the rounded weight, true when v is farther than
// the margin from a rounding boundary (else the double expression decides).
__device__ __forceinline__ bool nlink_fast(int d2, const NlinkParams &q, int &w) {
    const float v = q.lf * ex2_approx(-small_int_to_float(d2) * q.scale);
    if (q.small) {
        const float t = __fadd_rn(v, 12582912.0f);  // 1.5 * 2^23 + rint(v)
        const float rf = __fsub_rn(t, 12582912.0f);
        w = __float_as_int(t) - 0x4B400000;
        return fabsf(__fsub_rn(v, rf)) < q.half_margin;
    }
    const float fr = v - floorf(v);
    w = (int)floorf(v + 0.5f);
    return fabsf(fr - 0.5f) > q.margin;
}

__device__ __forceinline__ int nlink_quant(int d2, const NlinkParams &q) {
    int w;
    return nlink_fast(d2, q, w) ? w : nlink_exact(d2, q.lambda, q.s2);
}

// Aligned 32-bit word at a (a % 4 == 0) of the byte range [lo, hi): one load
// when the word lies inside, else the bytes inside and zeros elsewhere.
__device__ __forceinline__ uint32_t word_in(uintptr_t a, uintptr_t lo, uintptr_t hi) {
    if (a >= lo && a + 4 <= hi) return __ldg(reinterpret_cast<const uint32_t *>(a));
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (a + k >= lo && a + k < hi) w |= (uint32_t)__ldg(reinterpret_cast<const uint8_t *>(a + k)) << (8 * k);
    return w;
}

// The same for an aligned 16-byte vector (a % 16 == 0).
__device__ __forceinline__ uint4 vec_in(uintptr_t a, uintptr_t lo, uintptr_t hi) {
    if (a >= lo && a + 16 <= hi) return __ldg(reinterpret_cast<const uint4 *>(a));
    return make_uint4(word_in(a, lo, hi), word_in(a + 4, lo, hi), word_in(a + 8, lo, hi), word_in(a + 12, lo, hi));
}

// Bytes b of a word whose offsets o + b fall in [k0, k1) (32-bit offsets).
__device__ __forceinline__ uint32_t byte_mask(int o, int k0, int k1) {
    const int f = k0 - o, l = k1 - o;  // first and one-past-last valid byte
    const uint32_t upto_l = l <= 0 ? 0u : l >= 4 ? 0xFFFFFFFFu : (1u << (8 * l)) - 1u;
    const uint32_t upto_f = f <= 0 ? 0u : f >= 4 ? 0xFFFFFFFFu : (1u << (8 * f)) - 1u;
    return upto_l & ~upto_f;
}

__device__ __forceinline__ uint32_t sq4(uint32_t a, uint32_t b) {
    const uint32_t d = __vabsdiffu4(a, b);
    return __dp4a(d, d, 0u);
}

// Sum over the byte pairs of one chunk (see k_hist_sigma_b).  The chunk's
// bytes are offsets [0, L) relative to `c0` (its first byte); a lane takes
// the aligned 16-byte vector at aw + 16 v, v = lane, lane + 32, ...: its
// right partners (bytes + 3) come from itself and the next lane's first
// word, its down partners (bytes + 3W) from the two vectors at
// + (3W rounded down to 16) shifted by (3W mod 16) bytes: WS whole words
// and BS bytes, WS fixed per instantiation.  Byte k pairs right when
// k < kh and down when k < kv (chunk-relative).
template <int WS>
__device__ __forceinline__ uint32_t sigma_chunk(uintptr_t lo, uintptr_t hi, uintptr_t c0, uintptr_t aw, int nvec,
                                                uintptr_t vstep, int bs, int kh, int kv, uint4 *keep) {
    const int lane = threadIdx.x & 31;
    uint32_t acc = 0;  // at most 4 vectors of 32 pairs of 65025 per thread
    for (int v0 = (int)threadIdx.x - lane; v0 < nvec; v0 += blockDim.x) {  // warp-uniform trip count
        const int vi = v0 + lane;
        const uintptr_t a = aw + 16 * (uintptr_t)vi;
        // every lane loads (a lane past the end supplies its neighbour's next
        // vector); bytes outside the image read as 0
        uint4 c, u, u31 = make_uint4(0, 0, 0, 0);
        uint32_t c31 = 0;
        if (a >= lo && a + vstep + 32 <= hi) {
            c = __ldg(reinterpret_cast<const uint4 *>(a));
            u = __ldg(reinterpret_cast<const uint4 *>(a + vstep));
            if (lane == 31) {
                c31 = __ldg(reinterpret_cast<const uint32_t *>(a + 16));
                u31 = __ldg(reinterpret_cast<const uint4 *>(a + vstep + 16));
            }
        } else {
            c = vec_in(a, lo, hi);
            u = vec_in(a + vstep, lo, hi);
            if (lane == 31) {
                c31 = word_in(a + 16, lo, hi);
                u31 = vec_in(a + vstep + 16, lo, hi);
            }
        }
        uint32_t n0 = __shfl_down_sync(0xffffffffu, c.x, 1);
        uint32_t un[4];
        un[0] = __shfl_down_sync(0xffffffffu, u.x, 1);
        un[1] = WS >= 1 ? __shfl_down_sync(0xffffffffu, u.y, 1) : 0u;
        un[2] = WS >= 2 ? __shfl_down_sync(0xffffffffu, u.z, 1) : 0u;
        un[3] = WS >= 3 ? __shfl_down_sync(0xffffffffu, u.w, 1) : 0u;
        if (lane == 31) {
            n0 = c31;
            un[0] = u31.x;
            un[1] = u31.y;
            un[2] = u31.z;
            un[3] = u31.w;
        }
        if (vi < nvec) {
            keep[vi] = c;  // the chunk's colours, for the histogram pass
            const uint32_t cw[4] = {c.x, c.y, c.z, c.w};
            const uint32_t hw[5] = {c.x, c.y, c.z, c.w, n0};
            const uint32_t vw[8] = {u.x, u.y, u.z, u.w, un[0], un[1], un[2], un[3]};
            const int o = (int)(a - c0);  // chunk-relative offset of the vector's byte 0
            const bool full = o >= 0 && o + 16 <= kh && o + 16 <= kv;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                uint32_t dh = __vabsdiffu4(cw[j], __funnelshift_r(hw[j], hw[j + 1], 24));
                uint32_t dv = __vabsdiffu4(cw[j], __funnelshift_r(vw[j + WS], vw[j + WS + 1], bs));
                if (!full) {
                    dh &= byte_mask(o + 4 * j, 0, kh);
                    dv &= byte_mask(o + 4 * j, 0, kv);
                }
                acc += __dp4a(dh, dh, 0u) + __dp4a(dv, dv, 0u);
            }
        }
    }
    return acc;
}

// One pass over a chunk of an image (CHUNK_PX consecutive pixels, row-major):
// the exact sum of ||dI||^2 over right and down neighbour pairs (for sigma^2)
// and the scribble colour histograms (privatised per block in shared memory,
// equal bins of a warp aggregated with __match_any_sync before the shared
// atomics).
//
// The sum runs on the image's byte stream B (3 bytes per pixel, row-major):
// right pairs = sum of (B[k] - B[k + 3])^2 over the chunk's bytes k with
// k + 3 inside the image, minus the pairs that straddle a row end; down pairs
// = sum of (B[k] - B[k + 3W])^2 over the chunk's bytes above the image's last
// row.  Per 4 bytes: one __vabsdiffu4 + __dp4a for each direction.
// Eight blocks per SM (32 registers, 16 bytes of spills): the pass waits on
// memory, and the fuller SM hides more of it than six blocks with 40
// registers (batch256 0.130 -> 0.112 ms).
__global__ void __launch_bounds__(256, 8) k_hist_sigma_b(const uint8_t *__restrict__ rgb,
                                                      const uint8_t *__restrict__ scrib,
                                                      const ImgDesc *__restrict__ img,
                                                      const int2 *__restrict__ chunk_map,
                                                      int *__restrict__ hist, ImgState *ist) {
    __shared__ uint4 keep[(3 * CHUNK_PX + 15) / 16 + 1];  // the chunk's bytes from its 16-aligned start
    const int2 cm = __ldg(chunk_map + blockIdx.x);  // (image, chunk within the image)
    const int im = cm.x;
    const int W = img[im].W, H = img[im].H;
    const long long npx = (long long)W * H;
    const long long p0 = (long long)cm.y * CHUNK_PX;
    const int n = (int)min((long long)CHUNK_PX, npx - p0);  // pixels of the chunk
    const long long pix0 = img[im].pix0;
    const uint8_t *base = rgb + 3 * pix0;
    const bool do_hist = scrib != nullptr;
    const int lane = threadIdx.x & 31;
    unsigned long long acc = 0;
    {
        const long long W3 = 3LL * W, b0 = 3 * p0;
        const uintptr_t lo = (uintptr_t)base, hi = lo + (uintptr_t)(3 * npx);
        const uintptr_t c0 = lo + (uintptr_t)b0;
        const uintptr_t aw = c0 & ~(uintptr_t)15;
        const int L = 3 * n;
        const int nvec = (int)((c0 + L - aw + 15) >> 4);
        // chunk-relative limits: k + 3 inside the image; k + 3W inside the image
        const int kh = (int)min((long long)L, 3 * npx - 3 - b0);
        const int kv = (int)max(-1LL, min((long long)L, 3 * npx - W3 - b0));
        const uintptr_t vstep = (uintptr_t)(W3 & ~15LL);
        const int rem = (int)(W3 & 15);
        const int bs = (rem & 3) * 8;
        switch (rem >> 2) {
            case 0: acc = sigma_chunk<0>(lo, hi, c0, aw, nvec, vstep, bs, kh, kv, keep); break;
            case 1: acc = sigma_chunk<1>(lo, hi, c0, aw, nvec, vstep, bs, kh, kv, keep); break;
            case 2: acc = sigma_chunk<2>(lo, hi, c0, aw, nvec, vstep, bs, kh, kv, keep); break;
            default: acc = sigma_chunk<3>(lo, hi, c0, aw, nvec, vstep, bs, kh, kv, keep); break;
        }
        // right pairs that straddle a row end: rows y whose last pixel lies in
        // the chunk, below which another row follows
        const long long ya = (p0 + W) / W - 1, yb = min((p0 + n) / W - 1, (long long)H - 2);
        for (long long y = ya + threadIdx.x; y <= yb; y += blockDim.x) {
            const long long e = (y + 1) * W;  // first pixel of row y + 1
            acc -= sq4(pack_rgb(base + 3 * (e - 1)), pack_rgb(base + 3 * e));
        }
    }
    if (do_hist) {
        __syncthreads();  // the kept colours
        const uint8_t *kb = reinterpret_cast<const uint8_t *>(keep) + (int)(((uintptr_t)base + 3 * p0) & 15);
        int *dst = hist + (size_t)im * 2 * NBINS;
        // The chunk's scribble bytes, 16 per lane.  Scribbles come in short
        // runs (strips, squares), so a lane's 16 bytes are often all marked
        // while most lanes have none: the warp lists its marked bytes (a
        // prefix sum of the lanes' counts) and bins them 32 per round, lane k
        // taking item k of the list.  Equal bins of a round add once, with a
        // fire-and-forget global add.
        const uintptr_t slo = (uintptr_t)(scrib + pix0), shi = slo + (uintptr_t)npx;
        const uintptr_t s0 = slo + (uintptr_t)p0;
        const uintptr_t saw = s0 & ~(uintptr_t)15;
        const int nsv = (int)((s0 + n - saw + 15) >> 4);
        for (int v0 = (int)threadIdx.x - lane; v0 < nsv; v0 += blockDim.x) {
            const int vi = v0 + lane;
            const uintptr_t a = saw + 16 * (uintptr_t)vi;
            const uint4 sv = vi < nsv ? vec_in(a, slo, shi) : make_uint4(0, 0, 0, 0);
            const int o = (int)(a - s0);  // chunk pixel of the vector's byte 0
            // bit b: byte b is 1 or 2 and lies in the chunk (4 bytes at a time:
            // per-byte equality masks, then the bytes' top bits packed by a multiply)
            unsigned todo = 0;
            {
                const uint32_t sw[4] = {sv.x, sv.y, sv.z, sv.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    uint32_t m = __vcmpeq4(sw[j], 0x01010101u) | __vcmpeq4(sw[j], 0x02020202u);
                    if (o < 0 || o + 16 > n) m &= byte_mask(o + 4 * j, 0, n);
                    const uint32_t x = (m >> 7) & 0x01010101u;
                    todo |= ((x * 0x01020408u) >> 24) << (4 * j);
                }
            }
            const int cnt = __popc(todo);
            int incl = cnt;  // inclusive prefix sum of the counts over the warp
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            for (int r0 = 0; r0 < total; r0 += 32) {  // warp-uniform
                const int k = r0 + lane;
                // owner: the first lane whose inclusive sum exceeds k
                int lo = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int probe = __shfl_sync(0xffffffffu, incl, lo + step - 1);
                    if (probe <= k) lo += step;
                }
                const unsigned om = __shfl_sync(0xffffffffu, todo, lo);
                const int oincl = __shfl_sync(0xffffffffu, incl, lo);
                const int oo = __shfl_sync(0xffffffffu, o, lo);
                const uint32_t w0 = __shfl_sync(0xffffffffu, sv.x, lo), w1 = __shfl_sync(0xffffffffu, sv.y, lo);
                const uint32_t w2 = __shfl_sync(0xffffffffu, sv.z, lo), w3 = __shfl_sync(0xffffffffu, sv.w, lo);
                int key = -1;
                if (k < total) {
                    // the (k - owner's exclusive sum)-th marked byte of the owner
                    const int b = __fns(om, 0, k - (oincl - __popc(om)) + 1);
                    const uint32_t wb = b < 8 ? (b < 4 ? w0 : w1) : (b < 12 ? w2 : w3);
                    const int sc = (int)((wb >> (8 * (b & 3))) & 0xFFu);
                    const int q = oo + b;  // pixel of the chunk
                    const uint32_t col = (uint32_t)kb[3 * q] | ((uint32_t)kb[3 * q + 1] << 8) |
                                         ((uint32_t)kb[3 * q + 2] << 16);
                    key = (sc - 1) * NBINS + color_binw(col);
                }
                const unsigned same = __match_any_sync(0xffffffffu, key);
                if (key >= 0 && lane == __ffs(same) - 1) atomicAdd(dst + key, __popc(same));
            }
        }
    }
    warp_atomic_add_u64(&ist[im].sigma_sum, acc);
}

// Per-bin t-link tables (one block per image, double precision).
__global__ void __launch_bounds__(1024) k_tlut_b(const int *__restrict__ ilist, const int *__restrict__ hist,
                                                 int *__restrict__ dp_lut, int *__restrict__ dn_lut,
                                                 double *raw_dp, double *raw_dn) {
    __shared__ long long part[2][32];
    const int im = ilist ? ilist[blockIdx.x] : blockIdx.x;
    const int *hf = hist + (size_t)im * 2 * NBINS;
    const int *hb = hf + NBINS;
    long long nf = 0, nb = 0;
    for (int b = threadIdx.x; b < NBINS; b += blockDim.x) {
        nf += hf[b];
        nb += hb[b];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nf += __shfl_down_sync(0xffffffffu, nf, o);
        nb += __shfl_down_sync(0xffffffffu, nb, o);
    }
    if ((threadIdx.x & 31) == 0) {
        part[0][threadIdx.x >> 5] = nf;
        part[1][threadIdx.x >> 5] = nb;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        nf = threadIdx.x < (blockDim.x >> 5) ? part[0][threadIdx.x] : 0;
        nb = threadIdx.x < (blockDim.x >> 5) ? part[1][threadIdx.x] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nf += __shfl_down_sync(0xffffffffu, nf, o);
            nb += __shfl_down_sync(0xffffffffu, nb, o);
        }
        if (threadIdx.x == 0) {
            part[0][0] = nf;
            part[1][0] = nb;
        }
    }
    __syncthreads();
    const long long Nf = part[0][0] + NBINS, Nb = part[1][0] + NBINS;
    for (int b = threadIdx.x; b < NBINS; b += blockDim.x) {
        int qdp, qdn;
        if (raw_dp || raw_dn) {
            const double rdp = tlink_raw(hb[b], Nb), rdn = tlink_raw(hf[b], Nf);
            qdp = (int)round(rdp);
            qdn = (int)round(rdn);
            if (raw_dp) raw_dp[(size_t)im * NBINS + b] = rdp;
            if (raw_dn) raw_dn[(size_t)im * NBINS + b] = rdn;
        } else {
            qdp = tlink_quant(hb[b], Nb);
            qdn = tlink_quant(hf[b], Nf);
        }
        dp_lut[(size_t)im * NBINS + b] = qdp;
        dn_lut[(size_t)im * NBINS + b] = qdn;
    }
}

// N-link weight of a pair at squared colour distance d2 (s2 = sigma^2,
// 0 for a constant image, whose weights are all lambda).
__device__ __forceinline__ int nlink_w(int d2, const NlinkParams &q) {
    return q.constant ? q.const_w : nlink_quant(d2, q);
}

// Fused image -> residual graph of one tile: t-link gather, n-links, the
// reference's interior/border conventions, tile-major output.
//
// The tile's colours and a 1-pixel halo are staged in shared memory as packed
// words; every undirected edge between two interior pixels is weighed once
// (the weight is symmetric in its two pixels) into a right-edge and a
// down-edge table, and each pixel then reads its four capacities from them.
// An edge that touches the 1-pixel image border has capacity 0, as in the
// reference's graph (GraphCutKernels.cu:112-214).  Eight blocks per SM
// (32 registers, a few spilled): more tiles in flight hide the staging loads
// (batch256 0.426 ms at five blocks, 0.408 at six, 0.399 at eight).
__global__ void __launch_bounds__(TILE_THREADS, 8) k_build_img_b(Batch b, const uint8_t *__restrict__ rgb,
                                                               const int *__restrict__ dp_lut,
                                                               const int *__restrict__ dn_lut) {
    constexpr int SW = TILE_W + 2, SH = TILE_H + 2;
    __shared__ uint32_t col[SH][SW];              // pixel (x0 - 1 + j, y0 - 1 + i)
    __shared__ int wr[TILE_H][TILE_W + 1];        // edge (x, y)-(x + 1, y), x = x0 - 1 + j, y = y0 + i
    __shared__ int wd[TILE_H + 1][TILE_W];        // edge (x, y)-(x, y + 1), x = x0 + j, y = y0 - 1 + i
    const int t = batch_tile(b, blockIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int im = __ldg(b.tile_img + t);
    const ImgDesc d = b.img[im];
    const int lt = t - d.tile0;
    const int tx = lt % d.tiles_x, ty = lt / d.tiles_x;
    if (threadIdx.x == 0)  // the tile's neighbours, for the solver
        b.tile_nb[t] = make_int4(tx > 0 ? t - 1 : -1, tx < d.tiles_x - 1 ? t + 1 : -1, ty > 0 ? t - d.tiles_x : -1,
                                 ty < d.tiles_y - 1 ? t + d.tiles_x : -1);
    const int W = d.W, H = d.H;
    const int x0 = tx * TILE_W, y0 = ty * TILE_H;
    const NlinkParams q = nlink_params(d.lambda, b.ist[im]);
    const int *dpl = dp_lut + (size_t)im * NBINS;
    const int *dnl = dn_lut + (size_t)im * NBINS;
    const uint8_t *base = rgb + 3 * d.pix0;

    // Stage the 34 rows of 34 pixels (tile + 1-pixel halo) as packed colours.
    // Warp w takes rows w, w + 8, ...: the row's bytes are fetched as aligned
    // 32-bit words, one per lane (at most 27; a word that reaches outside
    // this image's bytes is assembled from the bytes inside), and each lane
    // cuts its pixel out of two adjacent words (warp shuffles + a funnel
    // shift); lanes 0 and 1 then cut the row's last two pixels.
    if (3LL * W * H < (1LL << 30)) {  // block-uniform: the image's byte offsets fit 32 bits
        // The same staging with 32-bit offsets from the 4-byte-aligned
        // address at or below the image's first byte (mis = the image's
        // misalignment): 64-bit address arithmetic costs several
        // instructions per operation, and every thread runs it per row.
        const uintptr_t lo = (uintptr_t)base;
        const int mis = (int)(lo & 3);
        const uint8_t *abase = base - mis;  // 4-byte aligned
        const int nbytes = 3 * W * H;
        const int xs = x0 > 0 ? x0 - 1 : 0;
        const int xe = x0 + TILE_W < W ? x0 + TILE_W : W - 1;
        constexpr int NW = TILE_THREADS / 32, RPW = (SH + NW - 1) / NW;  // rows per warp
        uint32_t words[RPW];
        int phs[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) {  // every load first
            const int i = warp + NW * r;
            const int y = y0 - 1 + i;
            uint32_t word = 0;
            const int rs = mis + 3 * (y * W + xs);  // aligned-base offset of the row's first byte
            phs[r] = rs & 3;
            if (i < SH && y >= 0 && y < H) {
                const int re = mis + 3 * (y * W + xe) + 3;  // one past its last byte
                const int aw = rs & ~3;
                if (lane < ((re - aw + 3) >> 2)) {
                    const int wa = aw + 4 * lane;   // aligned-base offset of the lane's word
                    const int k0 = wa - mis;        // image byte offset of its first byte
                    if (k0 >= 0 && k0 + 4 <= nbytes) {
                        word = __ldg(reinterpret_cast<const uint32_t *>(abase + wa));
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (k0 + k >= 0 && k0 + k < nbytes) word |= (uint32_t)__ldg(abase + wa + k) << (8 * k);
                    }
                }
            }
            words[r] = word;
        }
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const int i = warp + NW * r;
            if (i >= SH) break;  // warp-uniform
            const int y = y0 - 1 + i;
            const bool row_in = y >= 0 && y < H;
            const int ph = phs[r];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int j = lane + 32 * h;
                const int x = x0 - 1 + j;
                const bool in = row_in && x >= 0 && x < W;
                const int off = in ? ph + 3 * (x - xs) : 0;  // <= 3 + 3 * 33 = 102: words 0..26
                const uint32_t wlo = __shfl_sync(0xffffffffu, words[r], off >> 2);
                const uint32_t whi = __shfl_sync(0xffffffffu, words[r], (off >> 2) + 1);
                const uint32_t v = in ? __funnelshift_r(wlo, whi, (off & 3) * 8) & 0xFFFFFFu : 0u;
                if (j < SW) col[i][j] = v;
            }
        }
    } else {
        const uintptr_t lo = (uintptr_t)base, hi = lo + 3 * (uintptr_t)W * (uintptr_t)H;
        const int xs = x0 > 0 ? x0 - 1 : 0;
        const int xe = x0 + TILE_W < W ? x0 + TILE_W : W - 1;
        constexpr int NW = TILE_THREADS / 32, RPW = (SH + NW - 1) / NW;  // rows per warp
        uint32_t words[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) {  // every load first
            const int i = warp + NW * r;
            const int y = y0 - 1 + i;
            uint32_t word = 0;
            if (i < SH && y >= 0 && y < H) {
                const uintptr_t a0 = lo + 3 * ((uintptr_t)y * W + xs);
                const uintptr_t a1 = lo + 3 * ((uintptr_t)y * W + xe) + 3;
                const uintptr_t aw = a0 & ~(uintptr_t)3;
                if (lane < (int)((a1 - aw + 3) >> 2)) {
                    const uintptr_t wa = aw + 4 * (uintptr_t)lane;
                    if (wa >= lo && wa + 4 <= hi) {
                        word = __ldg(reinterpret_cast<const uint32_t *>(wa));
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (wa + k >= lo && wa + k < hi)
                                word |= (uint32_t)__ldg(reinterpret_cast<const uint8_t *>(wa + k)) << (8 * k);
                    }
                }
            }
            words[r] = word;
        }
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const int i = warp + NW * r;
            if (i >= SH) break;  // warp-uniform
            const int y = y0 - 1 + i;
            const bool row_in = y >= 0 && y < H;
            const int ph = (int)((lo + 3 * ((uintptr_t)y * W + xs)) & 3);  // first byte's place in its word
            // pixel j = lane (x = x0 - 1 + lane), then j = 32 + lane for lanes 0, 1
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int j = lane + 32 * h;
                const int x = x0 - 1 + j;
                const bool in = row_in && x >= 0 && x < W;
                const int off = in ? ph + 3 * (x - xs) : 0;  // <= 3 + 3 * 33 = 102: words 0..26
                const uint32_t wlo = __shfl_sync(0xffffffffu, words[r], off >> 2);
                const uint32_t whi = __shfl_sync(0xffffffffu, words[r], (off >> 2) + 1);
                const uint32_t v = in ? __funnelshift_r(wlo, whi, (off & 3) * 8) & 0xFFFFFFu : 0u;
                if (j < SW) col[i][j] = v;
            }
        }
    }
    __syncthreads();
    // 2048 edges inside the tile's rows and columns, 8 per thread (right
    // edges wr[i][1..32], then down edges wd[1..32][j]), and the 64 edges
    // that reach into the tile from the left and from above (wr[i][0], wd[0][j])
    {
        // thread (warp, lane): right edges of pixel (x0 + lane, y0 + warp + 8u),
        // u = 0..3, and down edges of the same pixels, u = 4..7
        constexpr int PER = 2 * TILE_W * TILE_H / TILE_THREADS;
        static_assert(PER == 8 && ROWS_PER_WARP == 4, "edge split assumes 8 warps of 32 lanes");
        const int x = x0 + lane;
        const bool xr = x >= 1 && x <= W - 3, xd = x >= 1 && x <= W - 2;
        // each weight goes to shared memory as soon as it is known; the rare
        // ones within the margin of a rounding boundary are redone exactly
        unsigned exact = 0;  // bit u: edge u needs the double expression
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int i = warp + 8 * (u & 3);
            const int y = y0 + i;
            bool use;
            int d2;
            if (u < 4) {
                use = xr && y >= 1 && y <= H - 2;
                d2 = diff2w(col[i + 1][lane + 1], col[i + 1][lane + 2]);
            } else {
                use = xd && y >= 1 && y <= H - 3;
                d2 = diff2w(col[i + 1][lane + 1], col[i + 2][lane + 1]);
            }
            int w = 0;
            if (q.constant) {
                w = q.const_w;
            } else if (!nlink_fast(d2, q, w)) {
                exact |= 1u << u;
            }
            if (!use) {
                w = 0;
                exact &= ~(1u << u);
            }
            if (u < 4) wr[i][lane + 1] = w;
            else wd[i + 1][lane] = w;
        }
        if (__any_sync(0xffffffffu, exact != 0)) {
            for (unsigned m = exact; m; m &= m - 1) {
                const int u = __ffs(m) - 1;
                const int i = warp + 8 * (u & 3);
                if (u < 4) wr[i][lane + 1] = nlink_exact(diff2w(col[i + 1][lane + 1], col[i + 1][lane + 2]), q.lambda, q.s2);
                else wd[i + 1][lane] = nlink_exact(diff2w(col[i + 1][lane + 1], col[i + 2][lane + 1]), q.lambda, q.s2);
            }
        }
        if (threadIdx.x < 2 * 32) {
            const int j = threadIdx.x & 31;
            int w = 0;
            if (threadIdx.x < 32) {  // edge (x0 - 1, y0 + j)-(x0, y0 + j)
                const int x = x0 - 1, y = y0 + j;
                if (x >= 1 && x <= W - 3 && y >= 1 && y <= H - 2) w = nlink_w(diff2w(col[j + 1][0], col[j + 1][1]), q);
                wr[j][0] = w;
            } else {  // edge (x0 + j, y0 - 1)-(x0 + j, y0)
                const int x = x0 + j, y = y0 - 1;
                if (y >= 1 && y <= H - 3 && x >= 1 && x <= W - 2) w = nlink_w(diff2w(col[0][j + 1], col[1][j + 1]), q);
                wd[0][j] = w;
            }
        }
    }
    __syncthreads();

    // Per pixel (thread (warp, lane), rows warp + 8k): capacities, excess and
    // the sums of the tile.  Per-thread sums stay below 2^30 (4 pixels of at
    // most GCFG_MAX_CAP), so they are 32-bit and each warp adds them exactly
    // with two 32-bit reductions of their 16-bit halves.
    __shared__ uint32_t msk[6][TILE_H];  // mask planes of the tile, stored coalesced below
    __shared__ unsigned long long wsum[3][TILE_THREADS / 32];
    const long long w32 = (long long)((W + 31) / 32) * 32, npx = (long long)W * H;
    const int x = x0 + lane;
    uint32_t idp = 0, rinit = 0, pos = 0;
    int4 *cap = b.cap + (size_t)t * TPX;
    int *exc = b.exc + (size_t)t * TPX;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const int y = y0 + r;
        int4 c = make_int4(0, 0, 0, 0);
        int e = 0;
        if (x < W && y < H) {
            const int bin = color_binw(col[r + 1][lane + 1]);
            const int vdp = __ldg(dpl + bin);
            if ((long long)x + (long long)y * w32 < npx && vdp > 0) rinit += (unsigned)vdp;
            if (x > 0 && y > 0 && x < W - 1 && y < H - 1) {
                c.x = wr[r][lane];      // left: edge (x - 1, y)-(x, y)
                c.y = wr[r][lane + 1];  // right
                c.z = wd[r][lane];      // up: edge (x, y - 1)-(x, y)
                c.w = wd[r + 1][lane];  // down
                e = vdp - __ldg(dnl + bin);
                idp += (unsigned)vdp;
            }
        }
        cap[r * 32 + lane] = c;
        exc[r * 32 + lane] = e;
        const unsigned ml = __ballot_sync(0xffffffffu, c.x > 0);
        const unsigned mr = __ballot_sync(0xffffffffu, c.y > 0);
        const unsigned mu = __ballot_sync(0xffffffffu, c.z > 0);
        const unsigned md = __ballot_sync(0xffffffffu, c.w > 0);
        const unsigned mn = __ballot_sync(0xffffffffu, e < 0);
        const unsigned mp = __ballot_sync(0xffffffffu, e > 0);
        if (lane == 0) {
            msk[0][r] = ml; msk[1][r] = mr; msk[2][r] = mu; msk[3][r] = md; msk[4][r] = mn; msk[5][r] = mp;
        }
        if (e > 0) pos += (unsigned)e;
    }
    {
        const uint32_t v[3] = {idp, rinit, pos};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const unsigned long long lo = __reduce_add_sync(0xffffffffu, v[k] & 0xFFFFu);
            const unsigned long long hi = __reduce_add_sync(0xffffffffu, v[k] >> 16);
            if (lane == 0) wsum[k][warp] = (hi << 16) + lo;
        }
    }
    __syncthreads();
    if (threadIdx.x < 6 * TILE_H)
        b.tmask[(size_t)t * 6 * 32 + threadIdx.x] = msk[threadIdx.x >> 5][threadIdx.x & 31];
    if (warp == 0) {
        // lanes 0..2: the tile's three sums
        unsigned long long tot = 0;
        if (lane < 3)
            for (int w8 = 0; w8 < TILE_THREADS / 32; ++w8) tot += wsum[lane][w8];
        if (lane == 0 && tot) atomicAdd(&b.ist[im].interior_dp, tot);
        if (lane == 1 && tot) atomicAdd(&b.ist[im].ref_init, tot);
        if (lane == 2) b.tile_pos[t] = tot;
    }
}

// Row-major t-link / n-link arrays of image 0 (the stand-alone data-term API).
__global__ void k_tlinks_apply(const uint8_t *__restrict__ rgb, long long n,
                               const int *__restrict__ dp_lut, const int *__restrict__ dn_lut,
                               int *__restrict__ dp, int *__restrict__ dn) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int bin = color_bin3(rgb + 3 * i);
    dp[i] = __ldg(dp_lut + bin);
    dn[i] = __ldg(dn_lut + bin);
}

__global__ void k_nlinks_apply(const uint8_t *__restrict__ rgb, const ImgDesc *__restrict__ img,
                               const ImgState *ist, int *__restrict__ up, int *__restrict__ down,
                               int *__restrict__ left, int *__restrict__ right) {
    const ImgDesc d = img[0];
    const int W = d.W, H = d.H;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const NlinkParams q = nlink_params(d.lambda, ist[0]);
    const long long i = (long long)y * W + x;
    const uint8_t *p = rgb + 3 * i;
    left[i] = x > 0 ? nlink_w(diff2p(p, p - 3), q) : 0;
    right[i] = x + 1 < W ? nlink_w(diff2p(p, p + 3), q) : 0;
    up[i] = y > 0 ? nlink_w(diff2p(p, p - 3 * (long long)W), q) : 0;
    down[i] = y + 1 < H ? nlink_w(diff2p(p, p + 3 * (long long)W), q) : 0;
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

gcfg_status dt_tables(const DtArgs &a, cudaStream_t st) {
    // a.scrib == NULL: n-link tables only (the colour histograms need scribbles)
    // (with an image list the caller clears the histograms of those images)
    if (a.scrib && !a.ilist) GCFG_CK(cudaMemsetAsync(a.hist, 0, (size_t)a.n_img * 2 * NBINS * sizeof(int), st));
    GCFG_LAUNCH(GCFG_PK_HIST, st,
                k_hist_sigma_b<<<a.total_chunks, 256, 0, st>>>(a.rgb, a.scrib, a.img, a.chunk_map, a.hist,
                                                               a.ist));
    GCFG_LAUNCH(GCFG_PK_TLUT, st, k_img_params<<<div_up(a.n_img, 128), 128, 0, st>>>(a.ilist, a.img, a.n_img, a.ist));
    if (a.scrib)
        GCFG_LAUNCH(GCFG_PK_TLUT, st,
                    k_tlut_b<<<a.n_img, 1024, 0, st>>>(a.ilist, a.hist, a.dp_lut, a.dn_lut, a.raw_dp, a.raw_dn));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status dt_build(const Batch &b, const DtArgs &a, cudaStream_t st) {
    GCFG_LAUNCH(GCFG_PK_BUILD, st,
                k_build_img_b<<<batch_ntiles(b), TILE_THREADS, 0, st>>>(b, a.rgb, a.dp_lut, a.dn_lut));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status dt_apply_tlinks(const DtArgs &a, long long n, int *dp, int *dn, cudaStream_t st) {
    GCFG_LAUNCH(GCFG_PK_OTHER, st,
                k_tlinks_apply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a.rgb, n, a.dp_lut, a.dn_lut, dp, dn));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status dt_apply_nlinks(const DtArgs &a, int W, int H, int *up, int *down, int *left, int *right,
                            cudaStream_t st) {
    dim3 blk(32, 8), grd(div_up(W, 32), div_up(H, 8));
    GCFG_LAUNCH(GCFG_PK_OTHER, st,
                k_nlinks_apply<<<grd, blk, 0, st>>>(a.rgb, a.img, a.ist, up, down, left, right));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

// Largest relative error of ex2_approx against the double 2^z over n
// evenly spaced z in [-64, 0] (the n-link fast path's error bound assumes
// <= 2^-21).  Relative errors are non-negative floats, so their bit
// patterns order like the values and an integer atomicMax finds the largest.
__global__ void k_selftest_ex2(long long n, int *max_bits) {
    float worst = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float z = -64.0f * (float)((double)i / (double)n);
        const double ref = exp2((double)z);
        const double rel = fabs((double)ex2_approx(z) - ref) / ref;
        worst = fmaxf(worst, (float)rel);
    }
    atomicMax(max_bits, __float_as_int(worst));
}

}  // namespace gcfg

extern "C" gcfg_status gcfg_selftest_ex2(int64_t samples, float *max_rel_err) {
    using namespace gcfg;
    if (samples < 1 || !max_rel_err) return GCFG_ERR_INVALID;
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
    int bits = 0;
    cudaError_t e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        k_selftest_ex2<<<1024, 256>>>((long long)samples, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&bits, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return GCFG_ERR_CUDA;
    memcpy(max_rel_err, &bits, sizeof(float));
    return GCFG_OK;
}
