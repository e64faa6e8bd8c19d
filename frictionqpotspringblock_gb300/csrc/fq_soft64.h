/*
 * IEEE-754 binary64 addition, subtraction and multiplication, rounded to nearest with ties to even,
 * computed with 32-bit integer instructions.
 *
 * Why: the step kernels are bound by the fp64 pipe, which on this GPU retires under two fp64
 * operations per clock per SM, while the 32-bit integer pipes (ALU and IMAD) sit mostly idle.
 * Issuing a share of a kernel's fp64 operations through these functions runs the pipes side by side.
 * The results are bit-identical to the hardware instruction for every input, so the arithmetic of the
 * step (and its parity with the reference) does not change.  Everything is written on 32-bit words:
 * 64-bit integer instructions would go back to the fp64 pipe on this GPU.
 *
 * Method (the definition of the format, nothing more): unpack sign, exponent and significand; for a
 * sum, align the smaller significand with a sticky bit, add or subtract, normalise; for a product,
 * form the 106-bit product of the significands from 32 x 32-bit partial products; round to nearest
 * even on the guard bits.  The fast path covers normal operands with a normal result; everything else
 * (zero, subnormal, infinite or NaN operands, a subnormal or overflowing result) is handed to the
 * hardware instruction in a branch that is not taken in practice.  The host build of the same source
 * (tests) checks the fast path against the host's IEEE arithmetic.
 */
#ifndef FQSB_FQ_SOFT64_H
#define FQSB_FQ_SOFT64_H

#include "fq_math.h"

#if defined(__CUDA_ARCH__)
/* Slow paths: not inlined, so the compiler branches around them instead of predicating an fp64
 * instruction into every call site. */
static __device__ __noinline__ double fq_s_hw_add(double a, double b)
{
    return __dadd_rn(a, b);
}
static __device__ __noinline__ double fq_s_hw_mul(double a, double b)
{
    return __dmul_rn(a, b);
}
FQ_HD uint32_t fq_s_lo(double x)
{
    return (uint32_t)__double2loint(x);
}
FQ_HD uint32_t fq_s_hi(double x)
{
    return (uint32_t)__double2hiint(x);
}
FQ_HD double fq_s_make(uint32_t hi, uint32_t lo)
{
    return __hiloint2double((int)hi, (int)lo);
}
/* (hi:lo) >> n, low word, n in [0, 32] */
FQ_HD uint32_t fq_s_shr64lo(uint32_t lo, uint32_t hi, uint32_t n)
{
    return __funnelshift_rc(lo, hi, n);
}
/* (hi:lo) << n, high word, n in [0, 32] */
FQ_HD uint32_t fq_s_shl64hi(uint32_t lo, uint32_t hi, uint32_t n)
{
    return __funnelshift_lc(lo, hi, n);
}
FQ_HD uint32_t fq_s_clz(uint32_t x)
{
    return (uint32_t)__clz((int)x);
}
/* (rh:rl) = (ah:al) + (bh:bl) mod 2^64, on 32-bit adds with carry */
FQ_HD void fq_s_add64(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t& rh, uint32_t& rl)
{
    asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, %4, %5;" : "=r"(rl), "=r"(rh) : "r"(al), "r"(bl), "r"(ah), "r"(bh));
}
FQ_HD void fq_s_sub64(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t& rh, uint32_t& rl)
{
    asm("sub.cc.u32 %0, %2, %3;\n\tsubc.u32 %1, %4, %5;" : "=r"(rl), "=r"(rh) : "r"(al), "r"(bl), "r"(ah), "r"(bh));
}
/* 64 x 64 -> 128-bit product of (ah:al) and (bh:bl) in 32-bit multiply-adds: p3:p2:p1:p0 */
FQ_HD void fq_s_mul128(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t& p3, uint32_t& p2, uint32_t& p1,
                       uint32_t& p0)
{
    asm("{\n\t"
        "mul.lo.u32     %0, %4, %6;\n\t"
        "mul.hi.u32     %1, %4, %6;\n\t"
        "mad.lo.cc.u32  %1, %5, %6, %1;\n\t"
        "madc.hi.u32    %2, %5, %6, 0;\n\t"
        "mad.lo.cc.u32  %1, %4, %7, %1;\n\t"
        "madc.hi.cc.u32 %2, %4, %7, %2;\n\t"
        "addc.u32       %3, 0, 0;\n\t"
        "mad.lo.cc.u32  %2, %5, %7, %2;\n\t"
        "madc.hi.u32    %3, %5, %7, %3;\n\t"
        "}"
        : "=&r"(p0), "=&r"(p1), "=&r"(p2), "=&r"(p3)
        : "r"(al), "r"(ah), "r"(bl), "r"(bh));
}
#define FQ_S_UNLIKELY(x) __builtin_expect(!!(x), 0)
#else
#if defined(FQ_S_COUNT_SLOW)
/* host checks count how often the hardware path was taken, to show the fast path is exercised */
extern long long fq_s_slow_count;
#define FQ_S_NOTE_SLOW() (++fq_s_slow_count)
#else
#define FQ_S_NOTE_SLOW() ((void)0)
#endif
static inline double fq_s_hw_add(double a, double b)
{
    FQ_S_NOTE_SLOW();
    return a + b;
}
static inline double fq_s_hw_mul(double a, double b)
{
    FQ_S_NOTE_SLOW();
    return a * b;
}
static inline uint32_t fq_s_lo(double x)
{
    return (uint32_t)fq_bits(x);
}
static inline uint32_t fq_s_hi(double x)
{
    return (uint32_t)(fq_bits(x) >> 32);
}
static inline double fq_s_make(uint32_t hi, uint32_t lo)
{
    return fq_from_bits(((uint64_t)hi << 32) | lo);
}
static inline uint32_t fq_s_shr64lo(uint32_t lo, uint32_t hi, uint32_t n)
{
    n = n > 32 ? 32 : n;
    return (uint32_t)((((uint64_t)hi << 32) | lo) >> n);
}
static inline uint32_t fq_s_shl64hi(uint32_t lo, uint32_t hi, uint32_t n)
{
    n = n > 32 ? 32 : n;
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << n) >> 32);
}
static inline uint32_t fq_s_clz(uint32_t x)
{
    return x ? (uint32_t)__builtin_clz(x) : 32u;
}
static inline void fq_s_add64(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t& rh, uint32_t& rl)
{
    uint64_t r = (((uint64_t)ah << 32) | al) + (((uint64_t)bh << 32) | bl);
    rh = (uint32_t)(r >> 32);
    rl = (uint32_t)r;
}
static inline void fq_s_sub64(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t& rh, uint32_t& rl)
{
    uint64_t r = (((uint64_t)ah << 32) | al) - (((uint64_t)bh << 32) | bl);
    rh = (uint32_t)(r >> 32);
    rl = (uint32_t)r;
}
static inline void fq_s_mul128(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t& p3, uint32_t& p2,
                               uint32_t& p1, uint32_t& p0)
{
    unsigned __int128 p = (unsigned __int128)((((uint64_t)ah << 32) | al)) * (((uint64_t)bh << 32) | bl);
    p0 = (uint32_t)p;
    p1 = (uint32_t)(p >> 32);
    p2 = (uint32_t)(p >> 64);
    p3 = (uint32_t)(p >> 96);
}
#define FQ_S_UNLIKELY(x) __builtin_expect(!!(x), 0)
#endif

/* Sum of (ah:al) and (bh:bl), the bit patterns of two doubles (b's sign already flipped for a
 * subtraction); a and b are the same values as doubles, for the hardware path. */
FQ_HD double fq_s_add_words(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, double a, double b)
{
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
    if (FQ_S_UNLIKELY(ea - 1u >= 0x7feu || eb - 1u >= 0x7feu)) {
        return fq_s_hw_add(a, b);
    }
    /* X: the operand of larger magnitude (sign of |A| - |B| from a 64-bit subtraction) */
    uint32_t dh, dl;
    fq_s_sub64(ah & 0x7fffffffu, al, bh & 0x7fffffffu, bl, dh, dl);
    (void)dl;
    const bool swap = (int32_t)dh < 0;
    const uint32_t xh = swap ? bh : ah, xl = swap ? bl : al;
    const uint32_t yh = swap ? ah : bh, yl = swap ? al : bl;
    const uint32_t ex = swap ? eb : ea, ey = swap ? ea : eb;
    /* significands with the implicit bit, moved up by 10 guard bits: leading bit at 62 */
    const uint32_t mxh = fq_s_shl64hi(xl, (xh & 0xfffffu) | 0x100000u, 10), mxl = xl << 10;
    uint32_t myh = fq_s_shl64hi(yl, (yh & 0xfffffu) | 0x100000u, 10), myl = yl << 10;
    /* align y by d = ex - ey (clamped to 63; y then only feeds the sticky bit) with a sticky bit */
    uint32_t d = ex - ey;
    d = d > 63u ? 63u : d;
    uint32_t sticky = 0;
    if (d >= 32u) {
        sticky = myl;
        myl = myh;
        myh = 0;
        d -= 32u;
    }
    sticky |= myl & ((1u << d) - 1u);
    myl = fq_s_shr64lo(myl, myh, d) | (sticky != 0u ? 1u : 0u);
    myh = myh >> d;
    /* add or subtract */
    uint32_t mh, ml;
    const bool sub = (int32_t)(xh ^ yh) < 0;
    if (sub) {
        fq_s_sub64(mxh, mxl, myh, myl, mh, ml);
    }
    else {
        fq_s_add64(mxh, mxl, myh, myl, mh, ml);
    }
    if ((mh | ml) == 0u) {
        return 0.0; /* exact cancellation: +0 when rounding to nearest */
    }
    /* normalise the leading bit to position 62: right by one on a carry, left after a cancellation */
    int32_t e = (int32_t)ex;
    if ((int32_t)mh < 0) {
        ml = fq_s_shr64lo(ml, mh, 1) | (ml & 1u);
        mh >>= 1;
        e += 1;
    }
    else {
        uint32_t lz = (mh != 0u ? fq_s_clz(mh) : 32u + fq_s_clz(ml)) - 1u;
        e -= (int32_t)lz;
        if (lz >= 32u) {
            mh = ml;
            ml = 0;
            lz -= 32u;
        }
        mh = fq_s_shl64hi(ml, mh, lz);
        ml = ml << lz;
    }
    if (FQ_S_UNLIKELY(e <= 0 || e >= 0x7ff)) {
        return fq_s_hw_add(a, b);
    }
    /* round to nearest even on the 10 guard bits: up when guard > half, or == half and lsb odd */
    uint32_t ql = fq_s_shr64lo(ml, mh, 10), qh = mh >> 10;
    const uint32_t up = ((ml & 0x3ffu) + 0x1ffu + (ql & 1u)) >> 10;
    fq_s_add64(qh, ql, 0u, up, qh, ql);
    /* the implicit bit (and a carry out of the significand) adds into the exponent field */
    return fq_s_make((xh & 0x80000000u) | (((uint32_t)(e - 1) << 20) + qh), ql);
}

FQ_HD double fq_sadd(double a, double b)
{
    return fq_s_add_words(fq_s_hi(a), fq_s_lo(a), fq_s_hi(b), fq_s_lo(b), a, b);
}

FQ_HD double fq_ssub(double a, double b)
{
    const uint32_t bh = fq_s_hi(b) ^ 0x80000000u;
    return fq_s_add_words(fq_s_hi(a), fq_s_lo(a), bh, fq_s_lo(b), a, fq_s_make(bh, fq_s_lo(b)));
}

FQ_HD double fq_smul(double a, double b)
{
    const uint32_t ah = fq_s_hi(a), al = fq_s_lo(a), bh = fq_s_hi(b), bl = fq_s_lo(b);
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
    if (FQ_S_UNLIKELY(ea - 1u >= 0x7feu || eb - 1u >= 0x7feu)) {
        return fq_s_hw_mul(a, b);
    }
    /* significands moved up by 11: leading bit at 63, product in [2^126, 2^128) */
    const uint32_t mah = fq_s_shl64hi(al, (ah & 0xfffffu) | 0x100000u, 11), mal = al << 11;
    const uint32_t mbh = fq_s_shl64hi(bl, (bh & 0xfffffu) | 0x100000u, 11), mbl = bl << 11;
    uint32_t p3, p2, p1, p0;
    fq_s_mul128(mah, mal, mbh, mbl, p3, p2, p1, p0);
    int32_t e = (int32_t)(ea + eb) - 1022;
    uint32_t lostw = p0 | p1;
    if ((int32_t)p3 >= 0) {
        p3 = fq_s_shl64hi(p2, p3, 1);
        p2 = fq_s_shl64hi(p1, p2, 1);
        lostw = p0 | (p1 << 1);
        e -= 1;
    }
    if (FQ_S_UNLIKELY(e <= 0 || e >= 0x7ff)) {
        return fq_s_hw_mul(a, b);
    }
    /* q = (p3:p2) >> 11; guard bits p2[10:0]; sticky: the words below */
    uint32_t ql = fq_s_shr64lo(p2, p3, 11), qh = p3 >> 11;
    const uint32_t g = p2 & 0x7ffu;
    const uint32_t up = (g + 0x3ffu + ((ql & 1u) | (lostw != 0u ? 1u : 0u))) >> 11;
    fq_s_add64(qh, ql, 0u, up, qh, ql);
    return fq_s_make(((ah ^ bh) & 0x80000000u) | (((uint32_t)(e - 1) << 20) + qh), ql);
}

#endif
