// Shared device helpers for the GB300 BGZF -> columns path.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

typedef uint64_t u64;
typedef unsigned int u32;
typedef unsigned short u16;
typedef unsigned char u8;

#define FRT_FULL_MASK 0xffffffffu
#define FRT_NONE64 0xffffffffffffffffull

// Per-member inflate status codes.  The numbering matches the reference
// kernel's FR_* codes (crates/fritillaria-cuda/kernels/inflate.cu:29-39) so a
// status means the same thing on both sides.
enum : u32 {
    INF_OK = 0,
    INF_TRUNCATED = 1,
    INF_BLOCK_TYPE = 2,
    INF_STORED_LEN = 3,
    INF_OUTPUT_OVERFLOW = 4,
    INF_BAD_CODE = 5,
    INF_BAD_DISTANCE = 6,
    INF_BAD_TABLE = 7,
    INF_BAD_LENGTH_REPEAT = 8,
    INF_BAD_COUNTS = 9,
    // not a reference code: a staging copy of the compressed member did not
    // complete within its bound (a device fault, not a property of the data)
    INF_STAGING_TIMEOUT = 10,
};

__device__ __forceinline__ u32 ld_u32le(const u8 *p)
{
    return (u32)p[0] | ((u32)p[1] << 8) | ((u32)p[2] << 16) | ((u32)p[3] << 24);
}
__device__ __forceinline__ u32 ld_u16le(const u8 *p) { return (u32)p[0] | ((u32)p[1] << 8); }

__device__ __forceinline__ u32 lane_id()
{
    u32 l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

__device__ __forceinline__ u32 lanemask_lt()
{
    u32 m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// CRC-32/ISO-HDLC (reflected 0xEDB88320).  Tables come from the polynomial;
// concatenation uses the GF(2) linearity crc(A||B) = crc(A)*x^(8|B|) + crc(B).
// ---------------------------------------------------------------------------
__device__ __forceinline__ u32 gf2_mulmod(u32 a, u32 b)
{
    u32 r = 0;
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
        r ^= b & (0u - (a >> 31));
        a <<= 1;
        b = (b >> 1) ^ (0xEDB88320u & (0u - (b & 1u)));
    }
    return r;
}

// x^(8 * 2^k) mod P for k = 0..31 (repeated squaring of x^8 in GF(2)[x]/P).
static __device__ const u32 c_crc_pow8[32] = {
    0x00800000u, 0x00008000u, 0xedb88320u, 0xb1e6b092u, 0xa06a2517u, 0xed627daeu, 0x88d14467u, 0xd7bbfe6au,
    0xec447f11u, 0x8e7ea170u, 0x6427800eu, 0x4d47bae0u, 0x09fe548fu, 0x83852d0fu, 0x30362f1au, 0x7b5a9cc3u,
    0x31fec169u, 0x9fec022au, 0x6c8dedc4u, 0x15d6874du, 0x5fde7a4eu, 0xbad90e37u, 0x2e4e5eefu, 0x4eaba214u,
    0xa8a472c0u, 0x429a969eu, 0x148d302au, 0xc40ba6d0u, 0xc4e22c3cu, 0x40000000u, 0x20000000u, 0x08000000u};

__device__ __forceinline__ u32 crc_shift(u32 crc, u64 nbytes)
{
    // crc * x^(8 n) mod P
    int k = 0;
    while (nbytes) {
        if (nbytes & 1ull) crc = gf2_mulmod(c_crc_pow8[k], crc);
        nbytes >>= 1;
        ++k;
    }
    return crc;
}

__device__ __forceinline__ u32 crc_combine(u32 crc_a, u32 crc_b, u64 len_b)
{
    return crc_shift(crc_a, len_b) ^ crc_b;
}
