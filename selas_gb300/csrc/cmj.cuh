// Correlated multi-jittered sampling: A. Kensler, "Correlated Multi-Jittered Sampling", Pixar Technical Memo
// 13-01 (2013), whose published hash constants and steps the reference's CorrelatedMultiJitter
// (Source/Core/MathLib/CorrelatedMultiJitter.cpp:12-62) uses; the deferred path tracer jitters sample s of pixel
// p by cmj_point(s, m, m, p) (Camera.cpp:77-86, DeferredPathTracer.cpp:349-380).  Integer hashing and IEEE
// float division only, so host and device give the same bits.
#pragma once

#include <cstdint>

#include "vecmath.cuh"

namespace sel {

// A bijection of [0, 2^k) (2^k the smallest power of two >= l) walked until it lands below l, then rotated by
// p: at most 2^k rounds.
SEL_HD uint32_t cmj_permute(uint32_t i, uint32_t l, uint32_t p) {
    uint32_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    for (uint32_t round = 0; round <= w; ++round) {
        i ^= p;
        i *= 0xe170893du;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3fu;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1u | p >> 27;
        i *= 0x6935fa69u;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303u;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3u;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfu;
        i &= w;
        i ^= i >> 5;
        if (i < l) break;
    }
    return (i + p) % l;
}

// Hash of (i, p) to [0, 1).
SEL_HD float cmj_float(uint32_t i, uint32_t p) {
    i ^= p;
    i ^= i >> 17;
    i ^= i >> 10;
    i *= 0xb36534e5u;
    i ^= i >> 12;
    i ^= i >> 21;
    i *= 0x93fc4795u;
    i ^= 0xdf6e307fu;
    i ^= i >> 17;
    i *= 1u | p >> 18;
    return float(i) * (1.0f / 4294967808.0f);
}

// Sample s of an m x n pattern decorrelated by p: a point of [0, 1)^2.
SEL_HD float2 cmj_point(int32_t s, int32_t m, int32_t n, int32_t p) {
    const uint32_t up = uint32_t(p);
    const int32_t sx = int32_t(cmj_permute(uint32_t(s % m), uint32_t(m), up * 0xa511e9b3u));
    const int32_t sy = int32_t(cmj_permute(uint32_t(s / m), uint32_t(n), up * 0x63d83595u));
    const float jx = cmj_float(uint32_t(s), up * 0xa399d265u);
    const float jy = cmj_float(uint32_t(s), up * 0x711ad6a5u);
    return make_float2((float(s % m) + (float(sy) + jx) / float(n)) / float(m),
                       (float(s / m) + (float(sx) + jy) / float(m)) / float(n));
}

}  // namespace sel
