// Batch compact encodings on the GPU (include/psy_gpu.h: psy_compact_*,
// psy_fluv32_decode_yuv, psy_color_compress / psy_color_decompress,
// psy_closure_compress / psy_closure_decompress).
//
// The codecs are HBM-bound byte work: 12 bytes of f32 triple in, 4 to 6
// bytes of code out (or back).  Work goes in tiles of 1024 elements: a
// tile's input bytes are staged in shared memory with 16-byte coalesced
// copies, converted element by element between two shared buffers, and
// written back with 16-byte coalesced stores, so that the 5- and 6-byte
// formats (whose elements straddle words) and the 12-byte triples cost no
// partial-sector traffic.  Read-heavy conversions with a 16-byte aligned
// input stream the tiles through resident blocks with the next tile's copy
// in flight during conversion; the rest take one tile per block (with
// byte-wise copies for pointers that are not 16-byte aligned; same results).  Elements outside
// a format's domain -- the inputs the reference's debug build rejects with
// an assertion -- are counted into an optional device counter.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/psy_gpu.h"
#include "dev_compact.cuh"

int psy_fail(int code, const std::string &msg);  // capi.cu: sets psy_last_error

namespace {

constexpr int kTile = 1024;    // elements per block
constexpr int kThreads = 256;  // threads per block

__device__ __forceinline__ void copy_bytes(uint8_t *__restrict__ dst, const uint8_t *__restrict__ src, uint32_t bytes,
                                           bool vec) {
    uint32_t done = 0;
    if (vec) {
        const uint32_t n16 = bytes / 16;
        for (uint32_t i = threadIdx.x; i < n16; i += kThreads)
            reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
        done = n16 * 16;
    }
    for (uint32_t i = done + threadIdx.x; i < bytes; i += kThreads) dst[i] = src[i];
}

__device__ __forceinline__ float3 ld3(const uint8_t *p) {
    const float *f = reinterpret_cast<const float *>(p);
    return make_float3(f[0], f[1], f[2]);
}
__device__ __forceinline__ void st3(uint8_t *p, float3 v) {
    float *f = reinterpret_cast<float *>(p);
    f[0] = v.x;
    f[1] = v.y;
    f[2] = v.z;
}
__device__ __forceinline__ void st_le(uint8_t *p, uint64_t v, int bytes) {
#pragma unroll
    for (int i = 0; i < 8; i++)
        if (i < bytes) p[i] = (uint8_t)(v >> (8 * i));
}
__device__ __forceinline__ uint64_t ld_le(const uint8_t *p, int bytes) {
    uint64_t v = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
        if (i < bytes) v |= (uint64_t)p[i] << (8 * i);
    return v;
}

// The domain the reference's encoders assert in debug builds.
__device__ __forceinline__ bool nonneg(float3 v) { return v.x >= 0.0f && v.y >= 0.0f && v.z >= 0.0f; }
__device__ __forceinline__ bool not_nan(float3 v) { return !isnan(v.x) && !isnan(v.y) && !isnan(v.z); }

// Element operations.  A packing op (kPack) reads one input record from the
// staged tile and returns its code (the low kOut bytes of a u64, as the
// crate lays them out little-endian), counting an element outside the
// format's domain into `bad`; an unpacking op gets one code and writes the
// output record.
template <int F>
struct Encode;
template <>
struct Encode<PSY_COMPACT_FLUV32> {
    static constexpr bool kPack = true;
    static constexpr int kIn = 12, kOut = 4;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &bad) {
        const float3 v = ld3(i);
        bad += !nonneg(v);
        return psyc::fluv32_encode(v.x, v.y, v.z);
    }
};
template <>
struct Encode<PSY_COMPACT_OCT32> {
    static constexpr bool kPack = true;
    static constexpr int kIn = 12, kOut = 4;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &) {
        const float3 v = ld3(i);
        return psyc::oct32_encode(v.x, v.y, v.z);
    }
};
template <>
struct Encode<PSY_COMPACT_OCT32_PRECISE> {
    static constexpr bool kPack = true;
    static constexpr int kIn = 12, kOut = 4;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &) {
        const float3 v = ld3(i);
        return psyc::oct32_encode_precise(v.x, v.y, v.z);
    }
};
template <>
struct Encode<PSY_COMPACT_UNSIGNED32> {
    static constexpr bool kPack = true;
    static constexpr int kIn = 12, kOut = 4;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &bad) {
        const float3 v = ld3(i);
        bad += !nonneg(v);
        return psyc::unsigned32_encode(v.x, v.y, v.z);
    }
};
template <>
struct Encode<PSY_COMPACT_UNSIGNED40> {
    static constexpr bool kPack = true;
    static constexpr int kIn = 12, kOut = 5;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &bad) {
        const float3 v = ld3(i);
        bad += !nonneg(v);
        return psyc::unsigned40_encode(v.x, v.y, v.z);
    }
};
template <>
struct Encode<PSY_COMPACT_SIGNED48> {
    static constexpr bool kPack = true;
    static constexpr int kIn = 12, kOut = 6;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &bad) {
        const float3 v = ld3(i);
        bad += !not_nan(v);
        return psyc::signed48_encode(v.x, v.y, v.z);
    }
};

template <int F>
struct Decode;
template <>
struct Decode<PSY_COMPACT_FLUV32> {
    static constexpr bool kPack = false;
    static constexpr int kIn = 4, kOut = 12;
    __device__ static uint32_t run(uint64_t c, uint8_t *o) {
        st3(o, psyc::fluv32_decode((uint32_t)c));
        return 0;
    }
};
template <>
struct Decode<PSY_COMPACT_OCT32> {
    static constexpr bool kPack = false;
    static constexpr int kIn = 4, kOut = 12;
    __device__ static uint32_t run(uint64_t c, uint8_t *o) {
        st3(o, psyc::oct32_decode((uint32_t)c));
        return 0;
    }
};
template <>
struct Decode<PSY_COMPACT_UNSIGNED32> {
    static constexpr bool kPack = false;
    static constexpr int kIn = 4, kOut = 12;
    __device__ static uint32_t run(uint64_t c, uint8_t *o) {
        st3(o, psyc::unsigned32_decode((uint32_t)c));
        return 0;
    }
};
template <>
struct Decode<PSY_COMPACT_UNSIGNED40> {
    static constexpr bool kPack = false;
    static constexpr int kIn = 5, kOut = 12;
    __device__ static uint32_t run(uint64_t c, uint8_t *o) {
        st3(o, psyc::unsigned40_decode(c));
        return 0;
    }
};
template <>
struct Decode<PSY_COMPACT_SIGNED48> {
    static constexpr bool kPack = false;
    static constexpr int kIn = 6, kOut = 12;
    __device__ static uint32_t run(uint64_t c, uint8_t *o) {
        st3(o, psyc::signed48_decode(c));
        return 0;
    }
};
// fluv32 to Y plus the two chroma bytes (fluv32.rs decode_yuv, :160-170)
struct DecodeYuv {
    static constexpr bool kPack = false;
    static constexpr int kIn = 4, kOut = sizeof(PsyYuv);
    __device__ static uint32_t run(uint64_t c64, uint8_t *o) {
        const uint32_t c = (uint32_t)c64;
        PsyYuv r;
        r.y = psyc::fluv32_y(c);
        r.u = (uint8_t)(c >> 8);
        r.v = (uint8_t)c;
        r.pad[0] = r.pad[1] = 0;
        *reinterpret_cast<PsyYuv *>(o) = r;
        return 0;
    }
};

// Colour (src/color.rs:144-249): one discriminant byte, then the fluv32 code
// of an XYZ colour (native-endian u32), or a blackbody / temperature colour's
// temperature as a saturating u16 and its factor as f16, little-endian: a
// 40-bit code, discriminant in the low byte.
__device__ __forceinline__ uint64_t color_code(const PsyColor &c, uint32_t &bad) {
    if (c.kind == PSY_COLOR_XYZ) {
        bad += !nonneg(make_float3(c.v[0], c.v[1], c.v[2]));
        return (uint64_t)psyc::fluv32_encode(c.v[0], c.v[1], c.v[2]) << 8;
    }
    if (c.kind == PSY_COLOR_BLACKBODY || c.kind == PSY_COLOR_TEMPERATURE) {
        const uint32_t t = psyc::sat_u32(fminf(c.v[0], 65535.0f));
        return c.kind | ((uint64_t)(t | (psyc::f32_to_f16_bits(c.v[1]) << 16)) << 8);
    }
    bad += 1;  // no such colour in the reference: written as zeros
    return 0;
}

__device__ __forceinline__ uint32_t color_from_code(uint64_t code, PsyColor &c) {
    const uint32_t tag = (uint32_t)code & 0xffu, w = (uint32_t)(code >> 8);
    if (tag == 0) {
        const float3 v = psyc::fluv32_decode(w);
        c.kind = PSY_COLOR_XYZ;
        c.v[0] = v.x;
        c.v[1] = v.y;
        c.v[2] = v.z;
        return 0;
    }
    c.v[2] = 0.0f;
    if (tag == 1 || tag == 2) {
        c.kind = tag;
        c.v[0] = (float)(w & 0xffffu);
        c.v[1] = psyc::f16_bits_to_f32(w >> 16);
        return 0;
    }
    c.kind = PSY_COLOR_XYZ;  // unreachable!() in the reference
    c.v[0] = c.v[1] = 0.0f;
    return 1;
}

struct ColorCompress {
    static constexpr bool kPack = true;
    static constexpr int kIn = sizeof(PsyColor), kOut = 5;
    __device__ static uint64_t run(const uint8_t *i, uint32_t &bad) {
        return color_code(*reinterpret_cast<const PsyColor *>(i), bad);
    }
};
struct ColorDecompress {
    static constexpr bool kPack = false;
    static constexpr int kIn = 5, kOut = sizeof(PsyColor);
    __device__ static uint32_t run(uint64_t c, uint8_t *o) { return color_from_code(c, *reinterpret_cast<PsyColor *>(o)); }
};

// Convert one staged tile of cnt elements from s_in into s_out.  Packed 5-
// and 6-byte codes move between the warps' registers and the staged tile as
// whole 32-bit words: a warp's 32 consecutive codes fill 8*kOut words, and
// each word is put together from the (at most two) codes it overlaps,
// fetched by shuffle; a code is read back from the two words it overlaps
// with a funnel shift.
template <class Op>
__device__ __forceinline__ void convert_tile(const uint8_t *__restrict__ s_in, uint8_t *__restrict__ s_out,
                                             uint32_t cnt, uint32_t &bad) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if constexpr (Op::kPack) {
        // word w = lane + 32 j of a warp's 32 codes starts in code e at byte
        // p (the same for every chunk): its low bytes are code e's bytes
        // p.., the rest (when p + 4 > kOut) code e + 1's first bytes
        constexpr uint32_t kWords = 8 * Op::kOut;  // words of 32 codes
        uint32_t we[2], wp[2];
#pragma unroll
        for (uint32_t j = 0; j < 2; j++) {
            const uint32_t b = 4 * (lane + 32 * j);
            we[j] = min(b / Op::kOut, 31u);
            wp[j] = b - (b / Op::kOut) * Op::kOut;
        }
        for (uint32_t base = warp * 32; base < cnt; base += kThreads) {  // warp-uniform bound
            const uint32_t k = base + lane;
            const uint64_t code = k < cnt ? Op::run(s_in + k * Op::kIn, bad) : 0;
            if constexpr (Op::kOut == 4) {
                if (k < cnt) reinterpret_cast<uint32_t *>(s_out)[k] = (uint32_t)code;
            } else {
                uint32_t *wout = reinterpret_cast<uint32_t *>(s_out + base * Op::kOut);
                const uint32_t lo = (uint32_t)code, hi = (uint32_t)(code >> 32);
#pragma unroll
                for (uint32_t j = 0; j < 2; j++) {
                    const uint32_t l0 = __shfl_sync(0xffffffffu, lo, we[j]);
                    const uint32_t h0 = __shfl_sync(0xffffffffu, hi, we[j]);
                    const uint32_t l1 = __shfl_sync(0xffffffffu, lo, min(we[j] + 1, 31u));
                    const uint32_t w = lane + 32 * j;
                    if (w < kWords) {
                        uint32_t v = __funnelshift_rc(l0, h0, 8 * wp[j]);  // (h0:l0) >> 8p, 8p <= 32
                        if (wp[j] + 4 > (uint32_t)Op::kOut) v |= l1 << (8 * (Op::kOut - wp[j]));
                        wout[w] = v;
                    }
                }
            }
        }
    } else {
        for (uint32_t k = threadIdx.x; k < cnt; k += kThreads) {
            uint64_t code;
            if constexpr (Op::kIn == 4) {
                code = reinterpret_cast<const uint32_t *>(s_in)[k];
            } else {
                const uint32_t b = k * Op::kIn, o = b & 3u;
                const uint32_t *w = reinterpret_cast<const uint32_t *>(s_in) + (b >> 2);
                const uint32_t w0 = w[0], w1 = w[1];
                const uint32_t hi = (w1 >> (8 * o)) & ((1u << (8 * (Op::kIn - 4))) - 1u);
                code = __funnelshift_r(w0, w1, 8 * o) | ((uint64_t)hi << 32);
            }
            bad += Op::run(code, s_out + k * Op::kOut);
        }
    }
}

// Block total of the per-thread counts into the optional counter: one
// atomic per block at most.  Called by every thread of the block.
__device__ __forceinline__ void count_invalid(uint32_t bad, uint32_t *invalid, uint32_t *s_bad) {
    bad = __reduce_add_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31u) == 0) s_bad[threadIdx.x >> 5] = bad;
    __syncthreads();
    if (invalid && threadIdx.x == 0) {
        uint32_t sum = 0;
#pragma unroll
        for (int i = 0; i < kThreads / 32; i++) sum += s_bad[i];
        if (sum) atomicAdd(invalid, sum);
    }
}

// Any alignment: one tile per block, byte-wise copies where a pointer is
// not 16-byte aligned.
template <class Op>
__global__ void __launch_bounds__(kThreads) k_compact(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                       uint32_t n, uint32_t *__restrict__ invalid, bool vin,
                                                       bool vout) {
    __shared__ __align__(16) uint8_t s_in[kTile * Op::kIn];
    __shared__ __align__(16) uint8_t s_out[kTile * Op::kOut];
    __shared__ uint32_t s_bad[kThreads / 32];
    const uint64_t first = (uint64_t)blockIdx.x * kTile;
    const uint32_t cnt = (uint32_t)min((uint64_t)kTile, (uint64_t)n - first);
    copy_bytes(s_in, in + first * Op::kIn, cnt * Op::kIn, vin);
    __syncthreads();
    uint32_t bad = 0;
    convert_tile<Op>(s_in, s_out, cnt, bad);
    __syncthreads();
    copy_bytes(out + first * Op::kOut, s_out, cnt * Op::kOut, vout);
    count_invalid(bad, invalid, s_bad);
}

// Start the asynchronous copy of `bytes` bytes (16-byte aligned source and
// destination) into shared memory: 16-byte cp.async per thread, the ragged
// end (bytes % 16) by plain loads.  Completion: cp.async.wait_group.
__device__ __forceinline__ void load_tile_async(uint8_t *dst, const uint8_t *src, uint32_t bytes) {
    const uint32_t n16 = bytes / 16;
    for (uint32_t i = threadIdx.x; i < n16; i += kThreads) {
        const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst + 16 * i);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + 16 * i) : "memory");
    }
    for (uint32_t i = n16 * 16 + threadIdx.x; i < bytes; i += kThreads) dst[i] = src[i];
}

// 16-byte aligned input: resident blocks walk the tiles (tile t, t + grid,
// ...) with the next tile's load in flight (cp.async into the other half
// of a double buffer) while the current one converts, so the read stream
// never waits on conversion.  Each cp.async group is waited for by the
// hardware (cp.async.wait_group), not by a spin loop.
template <class Op>
__global__ void __launch_bounds__(kThreads) k_compact_pipe(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                            uint32_t n, uint32_t *__restrict__ invalid, bool vout) {
    __shared__ __align__(16) uint8_t s_in[2][kTile * Op::kIn];
    __shared__ __align__(16) uint8_t s_out[kTile * Op::kOut];
    __shared__ uint32_t s_bad[kThreads / 32];
    const uint32_t tiles = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);
    uint32_t t = blockIdx.x;  // the launch has at most `tiles` blocks
    auto count = [&](uint32_t tile) { return (uint32_t)min((uint64_t)kTile, (uint64_t)n - (uint64_t)tile * kTile); };
    load_tile_async(s_in[0], in + (uint64_t)t * kTile * Op::kIn, count(t) * Op::kIn);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    uint32_t bad = 0, buf = 0;
    for (; t < tiles; t += gridDim.x) {
        const uint32_t nt = t + gridDim.x;
        if (nt < tiles) load_tile_async(s_in[buf ^ 1], in + (uint64_t)nt * kTile * Op::kIn, count(nt) * Op::kIn);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // tile t's group has landed
        __syncthreads();
        const uint32_t cnt = count(t);
        convert_tile<Op>(s_in[buf], s_out, cnt, bad);
        __syncthreads();
        copy_bytes(out + (uint64_t)t * kTile * Op::kOut, s_out, cnt * Op::kOut, vout);
        buf ^= 1;
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    count_invalid(bad, invalid, s_bad);
}

// Resident blocks per SM of k_compact_pipe<Op> times the SM count (per
// device, computed once).
template <class Op>
uint32_t pipe_grid() {
    static uint32_t grid[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!grid[dev]) {
        int sms = 0, per = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_compact_pipe<Op>, kThreads, 0) != cudaSuccess)
            return 0;
        grid[dev] = (uint32_t)(sms * (per > 0 ? per : 1));
    }
    return grid[dev];
}

bool misaligned(const void *p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) != 0; }

template <class Op>
int launch(const void *in, void *out, uint32_t n, uint32_t *invalid, void *stream, const char *what) {
    if (n == 0) return PSY_OK;
    if (!in || !out) return psy_fail(PSY_E_INVALID, std::string(what) + ": null buffer");
    if (misaligned(invalid, 4)) return psy_fail(PSY_E_INVALID, std::string(what) + ": counter not 4-byte aligned");
    const bool vin = ((uintptr_t)in & 15u) == 0, vout = ((uintptr_t)out & 15u) == 0;
    const uint32_t blocks = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);
    // read-heavy conversions (encoders, colour compression) stream through
    // resident blocks; write-heavy ones are fastest one tile per block
    const uint32_t resident = (vin && Op::kIn > Op::kOut) ? pipe_grid<Op>() : 0;
    if (resident)
        k_compact_pipe<Op><<<min(blocks, resident), kThreads, 0, (cudaStream_t)stream>>>(
            static_cast<const uint8_t *>(in), static_cast<uint8_t *>(out), n, invalid, vout);
    else
        k_compact<Op><<<blocks, kThreads, 0, (cudaStream_t)stream>>>(static_cast<const uint8_t *>(in),
                                                                      static_cast<uint8_t *>(out), n, invalid, vin,
                                                                      vout);
    if (cudaGetLastError() != cudaSuccess) return psy_fail(PSY_E_CUDA, std::string(what) + ": launch failed");
    return PSY_OK;
}

// Closures (src/shading/surface_closure.rs:157-253): one discriminant byte
// (Lambert 0, GGX 1, Emit 2); GGX then carries roughness and fresnel, each
// clamped to [0, 1] and stored as a truncated u16 fraction of 65535; the
// colour follows.  Records sit at a fixed stride (the way MicropolyBatch
// packs them, src/surface/micropoly_batch.rs:322-332), one thread each.
__device__ __forceinline__ uint32_t closure_tag(uint32_t shader_kind) {
    return shader_kind == PSY_SHADER_LAMBERT ? 0u : shader_kind == PSY_SHADER_GGX ? 1u : 2u;
}

__global__ void k_closure_compress(const PsyShaderDesc *__restrict__ in, uint32_t n, uint32_t stride,
                                   uint8_t *__restrict__ out, uint32_t *__restrict__ invalid) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t bad = 0;
    if (i < n) {
        const PsyShaderDesc s = in[i];
        uint8_t *o = out + (uint64_t)i * stride;
        const bool known = s.kind == PSY_SHADER_EMIT || s.kind == PSY_SHADER_LAMBERT || s.kind == PSY_SHADER_GGX;
        const uint32_t size = s.kind == PSY_SHADER_GGX ? 10u : 6u;
        if (!known || size > stride) {
            bad = 1;  // out_data shorter than compressed_size(): a panic in the reference
        } else {
            o[0] = (uint8_t)closure_tag(s.kind);
            uint8_t *oc = o + 1;
            if (s.kind == PSY_SHADER_GGX) {
                const uint32_t r = psyc::sat_u32(fminf(fmaxf(s.roughness, 0.0f), 1.0f) * 65535.0f);
                const uint32_t f = psyc::sat_u32(fminf(fmaxf(s.fresnel, 0.0f), 1.0f) * 65535.0f);
                st_le(o + 1, r | (f << 16), 4);
                oc = o + 5;
            }
            st_le(oc, color_code(s.color, bad), 5);
        }
    }
    if (invalid) {
        bad = __reduce_add_sync(0xffffffffu, bad);
        if ((threadIdx.x & 31) == 0 && bad) atomicAdd(invalid, bad);
    }
}

__global__ void k_closure_decompress(const uint8_t *__restrict__ in, uint32_t n, uint32_t stride,
                                     PsyShaderDesc *__restrict__ out, uint32_t *__restrict__ invalid) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t bad = 0;
    if (i < n) {
        const uint8_t *r = in + (uint64_t)i * stride;
        PsyShaderDesc s;
        s.roughness = 0.0f;
        s.fresnel = 0.0f;
        const uint32_t tag = r[0];
        if (tag == 1 && stride < 10) {
            bad = 1;
            s.kind = PSY_SHADER_EMIT;
            s.color = PsyColor{PSY_COLOR_XYZ, {0.0f, 0.0f, 0.0f}};
        } else if (tag == 1) {
            const uint32_t w = (uint32_t)ld_le(r + 1, 4);
            s.kind = PSY_SHADER_GGX;
            s.roughness = (float)(w & 0xffffu) * (1.0f / 65535.0f);
            s.fresnel = (float)(w >> 16) * (1.0f / 65535.0f);
            bad = color_from_code(ld_le(r + 5, 5), s.color);
        } else {
            s.kind = tag == 0 ? PSY_SHADER_LAMBERT : PSY_SHADER_EMIT;
            bad = color_from_code(ld_le(r + 1, 5), s.color) | (tag > 2 ? 1u : 0u);
        }
        out[i] = s;
    }
    if (invalid) {
        bad = __reduce_add_sync(0xffffffffu, bad);
        if ((threadIdx.x & 31) == 0 && bad) atomicAdd(invalid, bad);
    }
}

}  // namespace

// psy_compact_element_size (include/psy_gpu.h).
extern "C" int psy_compact_element_size(uint32_t format, uint32_t *bytes) {
    if (!bytes) return psy_fail(PSY_E_INVALID, "compact: null size pointer");
    switch (format) {
        case PSY_COMPACT_FLUV32:
        case PSY_COMPACT_OCT32:
        case PSY_COMPACT_OCT32_PRECISE:
        case PSY_COMPACT_UNSIGNED32: *bytes = 4; return PSY_OK;
        case PSY_COMPACT_UNSIGNED40: *bytes = 5; return PSY_OK;
        case PSY_COMPACT_SIGNED48: *bytes = 6; return PSY_OK;
        default: return psy_fail(PSY_E_INVALID, "compact: unknown format");
    }
}

// psy_compact_encode (include/psy_gpu.h).
extern "C" int psy_compact_encode(uint32_t format, const float *d_xyz, uint32_t n, void *d_out, uint32_t *d_invalid,
                                  void *stream) {
    switch (format) {
        case PSY_COMPACT_FLUV32:
            return launch<Encode<PSY_COMPACT_FLUV32>>(d_xyz, d_out, n, d_invalid, stream, "fluv32 encode");
        case PSY_COMPACT_OCT32:
            return launch<Encode<PSY_COMPACT_OCT32>>(d_xyz, d_out, n, d_invalid, stream, "oct32 encode");
        case PSY_COMPACT_OCT32_PRECISE:
            return launch<Encode<PSY_COMPACT_OCT32_PRECISE>>(d_xyz, d_out, n, d_invalid, stream,
                                                             "oct32 encode_precise");
        case PSY_COMPACT_UNSIGNED32:
            return launch<Encode<PSY_COMPACT_UNSIGNED32>>(d_xyz, d_out, n, d_invalid, stream, "unsigned32 encode");
        case PSY_COMPACT_UNSIGNED40:
            return launch<Encode<PSY_COMPACT_UNSIGNED40>>(d_xyz, d_out, n, d_invalid, stream, "unsigned40 encode");
        case PSY_COMPACT_SIGNED48:
            return launch<Encode<PSY_COMPACT_SIGNED48>>(d_xyz, d_out, n, d_invalid, stream, "signed48 encode");
        default: return psy_fail(PSY_E_INVALID, "compact: unknown format");
    }
}

// psy_compact_decode (include/psy_gpu.h).
extern "C" int psy_compact_decode(uint32_t format, const void *d_in, uint32_t n, float *d_xyz, void *stream) {
    switch (format) {
        case PSY_COMPACT_FLUV32:
            return launch<Decode<PSY_COMPACT_FLUV32>>(d_in, d_xyz, n, nullptr, stream, "fluv32 decode");
        case PSY_COMPACT_OCT32:
        case PSY_COMPACT_OCT32_PRECISE:
            return launch<Decode<PSY_COMPACT_OCT32>>(d_in, d_xyz, n, nullptr, stream, "oct32 decode");
        case PSY_COMPACT_UNSIGNED32:
            return launch<Decode<PSY_COMPACT_UNSIGNED32>>(d_in, d_xyz, n, nullptr, stream, "unsigned32 decode");
        case PSY_COMPACT_UNSIGNED40:
            return launch<Decode<PSY_COMPACT_UNSIGNED40>>(d_in, d_xyz, n, nullptr, stream, "unsigned40 decode");
        case PSY_COMPACT_SIGNED48:
            return launch<Decode<PSY_COMPACT_SIGNED48>>(d_in, d_xyz, n, nullptr, stream, "signed48 decode");
        default: return psy_fail(PSY_E_INVALID, "compact: unknown format");
    }
}

// psy_fluv32_decode_yuv (include/psy_gpu.h).
extern "C" int psy_fluv32_decode_yuv(const uint32_t *d_in, uint32_t n, PsyYuv *d_yuv, void *stream) {
    return launch<DecodeYuv>(d_in, d_yuv, n, nullptr, stream, "fluv32 decode_yuv");
}

// psy_color_compress (include/psy_gpu.h).
extern "C" int psy_color_compress(const PsyColor *d_colors, uint32_t n, uint8_t *d_out, uint32_t *d_invalid,
                                  void *stream) {
    return launch<ColorCompress>(d_colors, d_out, n, d_invalid, stream, "color compress");
}

// psy_color_decompress (include/psy_gpu.h).
extern "C" int psy_color_decompress(const uint8_t *d_in, uint32_t n, PsyColor *d_colors, uint32_t *d_invalid,
                                    void *stream) {
    return launch<ColorDecompress>(d_in, d_colors, n, d_invalid, stream, "color decompress");
}

// psy_closure_compress (include/psy_gpu.h).
extern "C" int psy_closure_compress(const PsyShaderDesc *d_closures, uint32_t n, uint32_t stride, uint8_t *d_out,
                                    uint32_t *d_invalid, void *stream) {
    if (stride < 6) return psy_fail(PSY_E_INVALID, "closure compress: stride below the 6-byte minimum record");
    if (n == 0) return PSY_OK;
    if (!d_closures || !d_out) return psy_fail(PSY_E_INVALID, "closure compress: null buffer");
    if (misaligned(d_closures, 4) || misaligned(d_invalid, 4))
        return psy_fail(PSY_E_INVALID, "closure compress: closures or counter not 4-byte aligned");
    k_closure_compress<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_closures, n, stride, d_out, d_invalid);
    if (cudaGetLastError() != cudaSuccess) return psy_fail(PSY_E_CUDA, "closure compress: launch failed");
    return PSY_OK;
}

// psy_closure_decompress (include/psy_gpu.h).
extern "C" int psy_closure_decompress(const uint8_t *d_in, uint32_t n, uint32_t stride, PsyShaderDesc *d_closures,
                                      uint32_t *d_invalid, void *stream) {
    if (stride < 6) return psy_fail(PSY_E_INVALID, "closure decompress: stride below the 6-byte minimum record");
    if (n == 0) return PSY_OK;
    if (!d_in || !d_closures) return psy_fail(PSY_E_INVALID, "closure decompress: null buffer");
    if (misaligned(d_closures, 4) || misaligned(d_invalid, 4))
        return psy_fail(PSY_E_INVALID, "closure decompress: closures or counter not 4-byte aligned");
    k_closure_decompress<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_in, n, stride, d_closures, d_invalid);
    if (cudaGetLastError() != cudaSuccess) return psy_fail(PSY_E_CUDA, "closure decompress: launch failed");
    return PSY_OK;
}
