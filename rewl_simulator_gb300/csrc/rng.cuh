// Random streams and acceptance thresholds of the REWL engine.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): every attempted flip owns one 32-bit word addressed by
// (walker key, attempt counter), so the lanes of a warp can draw the uniforms of
// a whole chunk of sites at once, independently of which flips get accepted.
//
// The reference accepts an uphill move when u < exp(-dg) with dg the float
// entropy change (src/REWL/wang_landau.hpp:68-73).  Here that test is rewritten
// as dg < -ln(u) with a deterministic float -ln (explicit IEEE roundings only,
// identical on host and device), and because logDoS is held as an int64 count of
// 2^-36 units, "float(d * 2^-36) < thr" becomes the integer test d < T(thr).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define REWL_HD __host__ __device__ __forceinline__
#else
#define REWL_HD inline
#endif

namespace rewl {

static constexpr int kLogdosBits = 36;                       // logDoS unit = 2^-36
static constexpr double kLogdosScale = 68719476736.0;        // 2^36

enum : uint32_t {
    kStreamWL = 0x574C0001u,      // per-attempt acceptance uniforms
    kStreamExchange = 0x45580002u,// pairing and exchange acceptance
    kStreamInit = 0x494E0003u,    // initial spins
    kStreamAdjust = 0x41440004u,  // start site of the walk into the window
};

struct Philox4 { uint32_t x, y, z, w; };

// Philox key of an instance from its seed: the SplitMix64 finaliser (Steele, Lea, Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014).  Walker keys are
// (key_lo ^ walker, key_hi); mixing first keeps instances whose seeds differ only in low bits
// from handing their walkers each other's streams.
REWL_HD uint64_t instance_key(uint64_t seed)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

REWL_HD uint32_t mulhi32(uint32_t a, uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

REWL_HD Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        Philox4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
    }
    return c;
}

// Word (ctr & 3) of the block at counter (ctr >> 2, stream, w3) under key (seed, uid).
REWL_HD uint32_t philox_word(uint64_t seed, uint32_t uid, uint64_t ctr, uint32_t stream, uint32_t w3 = 0)
{
    Philox4 c;
    c.x = (uint32_t)(ctr >> 2);
    c.y = (uint32_t)(ctr >> 34);
    c.z = stream;
    c.w = w3;
    const Philox4 r = philox4x32_10(c, (uint32_t)seed ^ uid, (uint32_t)(seed >> 32));
    const uint32_t k = (uint32_t)(ctr & 3);
    return k == 0 ? r.x : k == 1 ? r.y : k == 2 ? r.z : r.w;
}

REWL_HD int clz32(uint32_t v)
{
#if defined(__CUDA_ARCH__)
    return __clz(v);
#else
    return __builtin_clz(v);
#endif
}

REWL_HD float bits_to_float(uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f; __builtin_memcpy(&f, &b, 4); return f;
#endif
}

REWL_HD uint32_t float_to_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t b; __builtin_memcpy(&b, &f, 4); return b;
#endif
}

// Explicitly rounded float operations (never contracted into FMAs).
#if defined(__CUDA_ARCH__)
#define RW_FMUL(a, b) __fmul_rn(a, b)
#define RW_FADD(a, b) __fadd_rn(a, b)
#define RW_FSUB(a, b) __fsub_rn(a, b)
#define RW_FDIV(a, b) __fdiv_rn(a, b)
#define RW_FMA(a, b, c) __fmaf_rn(a, b, c)
#define RW_U2F(v) __uint2float_rn(v)
#define RW_I2F(v) __int2float_rn(v)
#else
#define RW_FMUL(a, b) ((a) * (b))
#define RW_FADD(a, b) ((a) + (b))
#define RW_FSUB(a, b) ((a) - (b))
#define RW_FDIV(a, b) ((a) / (b))
#define RW_FMA(a, b, c) __builtin_fmaf(a, b, c)
#define RW_U2F(v) ((float)(v))
#define RW_I2F(v) ((float)(v))
#endif

// -ln(u), u = (2*(x>>1)+1) * 2^-32.  For u > 1/sqrt(2) the exact 1 - u = d gives
// -ln u = 2 atanh(d/(2-d)); otherwise u = m 2^-k with m in [sqrt(1/2), sqrt(2)] and
// -ln u = k ln2 + 2 atanh((1-m)/(1+m)); atanh by its series through s^9.  Every
// float operation is explicitly rounded, so host and device agree bit for bit.
REWL_HD float neglog_u32(uint32_t x)
{
    const uint32_t v = x | 1u;
    float s;
    int k = 0;
    if (v > 0xB504F333u) {
        // u > 1/sqrt(2): 1 - u = (2^32 - v) 2^-32 is exact; -ln u = 2 atanh(d / (2 - d))
        const float d = RW_FMUL(RW_U2F(0u - v), 2.3283064365386963e-10f);
        s = RW_FDIV(d, RW_FSUB(2.0f, d));
    } else {
        const int e = 31 - clz32(v);
        float m = RW_U2F(v);
        m = RW_FMUL(m, bits_to_float((uint32_t)(127 - e) << 23));
        k = 32 - e;
        if (m > 1.41421354f) { m = RW_FMUL(m, 0.5f); k -= 1; }
        s = RW_FDIV(RW_FSUB(1.0f, m), RW_FADD(m, 1.0f));   // -ln m = 2 atanh((1-m)/(1+m))
    }
    const float s2 = RW_FMUL(s, s);
    float p = RW_FMA(s2, 0.111111112f, 0.142857149f);
    p = RW_FMA(p, s2, 0.200000003f);
    p = RW_FMA(p, s2, 0.333333343f);
    p = RW_FMA(p, s2, 1.0f);
    const float q = RW_FMUL(RW_FMUL(2.0f, s), p);
    return RW_FMA(RW_I2F(k), 0.693147182f, q);
}

// Smallest integer d >= 1 with float(d * 2^-36) >= thr (thr > 0, finite, normal):
// for any int64 d, float(d * 2^-36) < thr  <=>  d < accept_threshold(thr).
// thr = m 2^e; the rounding boundary below thr is (2m-1) 2^(e-1) (ties to the
// even neighbour), or (4m-1) 2^(e-2) when thr is a power of two.
REWL_HD int64_t accept_threshold(float thr)
{
    const uint32_t b = float_to_bits(thr);
    const int be = (int)((b >> 23) & 0xFFu);
    const int64_t m = (int64_t)((b & 0x7FFFFFu) | 0x800000u);
    const int e = be - 150;
    int64_t A; int s; bool inclusive;
    if (m == 0x800000) { A = 4 * m - 1; s = e - 2; inclusive = true; }
    else { A = 2 * m - 1; s = e - 1; inclusive = (m & 1) == 0; }
    const int sh = s + kLogdosBits;
    if (sh >= 0) {
        if (sh > 62 - 26) return INT64_MAX;
        const int64_t D = A << sh;
        return inclusive ? D : D + 1;
    }
    if (-sh > 62) return 1;
    return (A >> (-sh)) + 1;
}

} // namespace rewl
