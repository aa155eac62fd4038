// Philox4x32-10 counter-based generator, written from the published description
// (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11):
// ten rounds, each two 32x32->64-bit multiplies by the round multipliers with the key mixed
// into the high halves, the key bumped by the Weyl constants between rounds.
// Usable from host and device code.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define TDS_HD __host__ __device__ __forceinline__
#else
#define TDS_HD inline
#endif

namespace tdsr {

TDS_HD void philox_round(uint32_t c[4], uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    const uint32_t o0 = hi1 ^ c[1] ^ k0, o2 = hi0 ^ c[3] ^ k1;
    c[0] = o0;
    c[1] = lo1;
    c[2] = o2;
    c[3] = lo0;
}

TDS_HD void philox10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k0 = key[0], k1 = key[1];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        philox_round(c, k0, k1);
    }
    out[0] = c[0], out[1] = c[1], out[2] = c[2], out[3] = c[3];
}

// The per-particle, per-step noise draw: counter (step lo, step hi, local id, replica),
// key = seed. Returns the top 24 bits of word 0, i.e. u * 2^24 for u uniform in [0,1).
TDS_HD uint32_t noise_bits24(uint64_t seed, int64_t step, uint32_t local, uint32_t rep) {
    const uint32_t ctr[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), local, rep};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    philox10(ctr, key, o);
    return o[0] >> 8;
}

}  // namespace tdsr
