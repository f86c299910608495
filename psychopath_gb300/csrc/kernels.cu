// Kernels of the GB300 tracing path: camera ray generation, the light-path
// state machine and accumulation (traversal kernels: trace_kernels.cu; the
// f32 camera and hit-shading kernels of the optimized form: wave_f32.cu).
#include <cuda_fp16.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "dev_bins.cuh"
#include "dev_surface.cuh"
#include "kernels.cuh"
#include "radix_sort.h"
#include "wave_kernels.cuh"

using namespace psyd;

// ------------------------------------------------------------------ constants
// Sobol direction numbers: dimension 1 is van der Corput, dimensions 2..8
// follow Joe & Kuo's primitive polynomials and initial direction numbers.
static void sobol_dirs_host(uint32_t d[8][32]) {
    static const uint32_t s_[7] = {1, 2, 3, 3, 4, 4, 5};
    static const uint32_t a_[7] = {0, 1, 1, 2, 1, 4, 2};
    static const uint32_t m_[7][5] = {{1}, {1, 3}, {1, 3, 1}, {1, 1, 1}, {1, 1, 3, 3}, {1, 3, 5, 13}, {1, 1, 5, 5, 17}};
    for (int k = 0; k < 32; k++) d[0][k] = 1u << (31 - k);
    for (int j = 1; j < 8; j++) {
        uint32_t s = s_[j - 1], a = a_[j - 1];
        for (uint32_t k = 0; k < 32; k++) {
            if (k < s) {
                d[j][k] = m_[j - 1][k] << (31 - k);
            } else {
                uint32_t x = d[j][k - s] ^ (d[j][k - s] >> s);
                for (uint32_t i = 1; i < s; i++)
                    if ((a >> (s - 1 - i)) & 1u) x ^= d[j][k - i];
                d[j][k] = x;
            }
        }
    }
}
// Child visit order per ray octant and node topology (sub_crates/bvh_order).
static void traversal_table_host(uint8_t t[8][48]) {
    for (int rd = 0; rd < 8; rd++) {
        int ray[3] = {rd & 1, (rd >> 1) & 1, (rd >> 2) & 1};
        int k = 0;
        auto sw = [](int &a, int &b) { int x = a; a = b; b = x; };
        for (int s2 = 0; s2 < 3; s2++)
            for (int s1 = 0; s1 < 3; s1++)
                for (int s0 = 0; s0 < 3; s0++) {
                    int p[4] = {0, 1, 2, 3};
                    if (ray[s1]) sw(p[0], p[1]);
                    if (ray[s2]) sw(p[2], p[3]);
                    if (ray[s0]) { sw(p[0], p[2]); sw(p[1], p[3]); }
                    t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2) | (p[2] << 4) | (p[3] << 6));
                }
        for (int s1 = 0; s1 < 3; s1++)
            for (int s0 = 0; s0 < 3; s0++) {
                int p[3] = {0, 1, 2};
                if (ray[s1]) sw(p[0], p[1]);
                if (ray[s0]) { sw(p[0], p[1]); sw(p[0], p[2]); }
                t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2) | (p[2] << 4));
            }
        for (int s1 = 0; s1 < 3; s1++)
            for (int s0 = 0; s0 < 3; s0++) {
                int p[3] = {0, 1, 2};
                if (ray[s1]) sw(p[1], p[2]);
                if (ray[s0]) { sw(p[0], p[2]); sw(p[0], p[1]); }
                t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2) | (p[2] << 4));
            }
        for (int s0 = 0; s0 < 3; s0++) {
            int p[2] = {0, 1};
            if (ray[s0]) sw(p[0], p[1]);
            t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2));
        }
    }
}
// Device copy of the table: positions past a node's child count (entries
// 27..44 order three children, 45..47 two) point at the node's empty child
// slots, so traversal can walk all four positions.
static void extend_traversal_table(uint8_t t[8][48]) {
    for (int rd = 0; rd < 8; rd++)
        for (int k = 27; k < 48; k++) {
            if (k < 45) t[rd][k] = (uint8_t)(t[rd][k] | (3u << 6));
            else t[rd][k] = (uint8_t)(t[rd][k] | (2u << 4) | (3u << 6));
        }
}
void psy_traversal_table_device(uint8_t t[8][48]) {
    traversal_table_host(t);
    extend_traversal_table(t);
}
// The nibble tables of the Sobol generator matrices (see g_sobol_nib).
static void sobol_nibble_tables(uint32_t nib[8][8][16]) {
    uint32_t d[8][32];
    sobol_dirs_host(d);
    for (int dim = 0; dim < 8; dim++)
        for (int p = 0; p < 8; p++)
            for (uint32_t v = 0; v < 16; v++) {
                uint32_t x = 0;
                for (int j = 0; j < 4; j++)
                    if ((v >> j) & 1u) x ^= d[dim][4 * p + j];
                nib[dim][p][v] = x;
            }
}
void psy_upload_constants() {
    static uint32_t nib[8][8][16];
    uint8_t t[8][48];
    sobol_nibble_tables(nib);
    psy_traversal_table_device(t);
    cudaMemcpyToSymbol(g_sobol_nib, nib, sizeof(nib));
    cudaMemcpyToSymbol(c_traversal_table, t, sizeof(t));
    psy_upload_trace_constants(t, nullptr);
    psy_upload_wave_f32_constants(nib, nullptr);
}

cudaError_t launch_camera(const GScene &S, const WaveDesc *d_wave, uint32_t max_paths, PathState P, RayBuf R,
                          uint32_t *queue, uint32_t *count, int prec, cudaStream_t st) {
    uint32_t n = max_paths;
    if (n == 0) return cudaSuccess;
    if (prec == 1) return launch_camera_f32(S, d_wave, n, P, R, queue, count, st);
    k_camera<double><<<(n + 255) / 256, 256, 0, st>>>(S, d_wave, P, R, queue, count);
    return cudaGetLastError();
}


// Shadow-ray results: the pending light contribution when the shadow ray
// was not occluded, then the next bounce ray if the path has one.
__global__ void __launch_bounds__(128, 12) k_shade_shadow(PathState P, RayBuf R, HitBuf H,
                                                         const uint32_t *__restrict__ queue,
                                                         const uint32_t *__restrict__ count, QueueOut out) {
    uint32_t n = *count;
    if (blockIdx.x * blockDim.x >= n) return;
    uint32_t stride = gridDim.x * blockDim.x;
    uint32_t nloop = (n + stride - 1) / stride * stride;  // keep whole warps in the loop for the ballot
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nloop; q += stride) {
        bool alive = false;
        uint32_t p = 0, key = 0;
        uint32_t fl = 0;
        if (q < n) {
            p = queue[q];
            fl = P.flags[p];
        }
        if (q < n && (fl & 3u) == EV_SHADOW) {
            uint32_t ev = fl & 3u, bounce = (fl >> 2) & 0xFFu, has_nb = (fl >> 10) & 1u, nrays = fl >> 16;
            nrays += 1;
            uint32_t kind = H.ki[p].x;
            if (kind == PSY_HIT_MISS_K) {
                V4 color = v4(P.color[p]) + v4(P.pending[p]);
                P.color[p] = f4(color);
            }
            if (has_nb) {
                float time = P.tw[p].x;
                float4 nb = P.nb_o[p], nd = P.nb_d[p];
                R.o[p] = make_float4(nb.x, nb.y, nb.z, CUDART_INF_F);
                R.d[p] = make_float4(nd.x, nd.y, nd.z, time);
                R.occl[p] = 0;  // the stored attenuation is already the bounce's
                ev = EV_BOUNCE;
                alive = true;
                if (out.keys) key = next_ray_key(out, v3(nb), v3(nd), false);
            }
            P.flags[p] = ev | (bounce << 2) | (has_nb << 10) | (nrays << 16) | PSY_SHADED_BIT;
        }
        push_live(alive, p, key, out);
    }
}

int queue_grid(const void *fn, int grid, uint32_t max_count) {
    int need = (int)((max_count + 127) / 128);
    if (grid > 0 || need == 0) return grid > 0 ? grid : 0;
    if (grid == 0) return need;
    const int rounds = -grid;  // -k: k rounds of the resident blocks
    // resident blocks of fn: SMs x blocks per SM at 128 threads, cached per
    // kernel and device (the query is a driver call)
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({fn, dev});
    if (it == cache.end()) {
        int sms = 0, per = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 128, 0);
        it = cache.emplace(std::make_pair(fn, dev), std::max(1, sms) * std::max(1, per)).first;
    }
    return (int)std::min<int64_t>(need, (int64_t)rounds * it->second);
}

cudaError_t launch_shade(const GScene &S, const WaveDesc *d_wave, PathState P, RayBuf R, HitBuf H, const uint32_t *queue,
                         const uint32_t *count, uint32_t max_count, const QueueOut &out, int minb, int grid, int prec,
                         cudaStream_t st) {
    int gs = queue_grid((const void *)k_shade_shadow, grid, max_count);
    if (gs == 0) return cudaSuccess;
    k_shade_shadow<<<gs, 128, 0, st>>>(P, R, H, queue, count, out);
#define SH(RT, MB)                                                                                           \
    {                                                                                                        \
        int g = queue_grid((const void *)k_shade_hit<RT, MB>, grid, max_count);                              \
        k_shade_hit<RT, MB><<<g, 128, 0, st>>>(S, d_wave, P, R, H, queue, count, out);                       \
    }
    // budget 4: the compiler's own choice in the f64 form (MINB 0 = unspecified,
    // ~154 registers), at most 128 registers in the f32 form (wave_f32.cu)
    if (prec == 1) return launch_shade_hit_f32(S, d_wave, P, R, H, queue, count, max_count, out, minb, grid, st);
    if (minb >= 8) SH(double, 8)
    else if (minb >= 6) SH(double, 6)
    else SH(double, 0)
#undef SH
    return cudaGetLastError();
}

// ------------------------------------------------------------------ queue binning
// Between wavefront iterations the live paths can be grouped by their next
// ray so that a warp's rays start near each other and point into the same
// octant: key = occlusion flag, direction octant, then a Morton code of the
// origin's cell (k bits per axis of the scene box), `bits` = 4 + 3k bits in
// all.  A counting sort (order inside a bin arbitrary); paths are
// independent, so the image does not change.  Wider keys (19, 25, 31 bits)
// use the two-point key of the trace calls' ray order, computed by the
// shading kernels as they write each live path's next ray (QueueOut), and a
// stable radix sort (radix_sort.cu).
__device__ __forceinline__ uint32_t queue_key(const GScene &S, float4 o, float4 d, bool occl, int bits) {
    uint32_t key = (occl ? 1u : 0u) | (ray_code(v3(d)) << 1);
    int per = (bits - 4) / 3;
    if (per > 0) {
        float cells = (float)(1u << per);
        uint32_t c[3];
        float ov[3] = {o.x, o.y, o.z}, lo[3] = {S.bounds_min.x, S.bounds_min.y, S.bounds_min.z},
              iv[3] = {S.bounds_inv_extent.x, S.bounds_inv_extent.y, S.bounds_inv_extent.z};
#pragma unroll
        for (int a = 0; a < 3; a++) c[a] = (uint32_t)fminf(fmaxf((ov[a] - lo[a]) * iv[a] * cells, 0.0f), cells - 1.0f);
        uint32_t m = 0;
        for (int b = 0; b < per; b++)
            m |= (((c[0] >> b) & 1u) << (3 * b)) | (((c[1] >> b) & 1u) << (3 * b + 1)) | (((c[2] >> b) & 1u) << (3 * b + 2));
        key |= m << 4;
    }
    return key;
}
__global__ void k_queue_keys(GScene S, RayBuf R, const uint32_t *__restrict__ queue, const uint32_t *__restrict__ count,
                             int bits, uint16_t *__restrict__ keys, uint32_t *__restrict__ hist) {
    uint32_t n = *count;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t q = base + threadIdx.x;
        uint32_t active = __ballot_sync(0xffffffffu, q < n);
        if (q < n) {
            uint32_t p = queue[q];
            uint32_t key = queue_key(S, R.o[p], R.d[p], R.occl[p] != 0, bits);
            keys[q] = (uint16_t)key;
            warp_add_key(hist, key, active);
        }
    }
}
__global__ void k_queue_scatter(const uint32_t *__restrict__ queue, const uint32_t *__restrict__ count,
                                const uint16_t *__restrict__ keys, uint32_t *__restrict__ cursor,
                                uint32_t *__restrict__ out, uint32_t *__restrict__ out_count) {
    uint32_t n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0) *out_count = n;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t q = base + threadIdx.x;
        uint32_t active = __ballot_sync(0xffffffffu, q < n);
        if (q < n) out[warp_add_key(cursor, keys[q], active)] = queue[q];
    }
}

size_t queue_radix_words(uint32_t n) { return 3 * (size_t)n + radix_sort_scratch_words(n); }

cudaError_t launch_queue_radix(const QueueSortBufs &Q, uint32_t *vals, const uint32_t *count, uint32_t max_count,
                               int bits, uint32_t **sorted, cudaStream_t st) {
    const int passes = (bits + 7) / 8;  // each pass moves (keys, vals) to the other buffer pair
    *sorted = (passes & 1) ? Q.vals2 : vals;
    return radix_sort_pairs_dev(Q.keys, vals, Q.keys2, Q.vals2, Q.scratch, count, max_count, bits, st);
}

cudaError_t launch_queue_binning(const GScene &S, RayBuf R, const uint32_t *queue, const uint32_t *count,
                                 uint32_t max_count, int bits, const QueueSortBufs &Q, uint32_t *out,
                                 uint32_t *out_count, cudaStream_t st) {
    int g = (int)std::min<uint32_t>((max_count + 255) / 256, 152u * 16u);
    if (g < 1) g = 1;
    if (bits > 16) return cudaErrorInvalidValue;  // radix-sorted keys come from the shading kernels
    uint32_t nbins = 1u << bits;
    cudaError_t e = cudaMemsetAsync(Q.bins, 0, nbins * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_queue_keys<<<g, 256, 0, st>>>(S, R, queue, count, bits, Q.keys16, Q.bins);
    k_scan_bins<<<1, 1024, 0, st>>>(Q.bins, nbins);
    k_queue_scatter<<<g, 256, 0, st>>>(queue, count, Q.keys16, Q.bins, out, out_count);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ spectrum tables
// One block per indexed colour, one thread per sample (see meng_table_value).
__global__ void k_spectrum_tables(const float4 *__restrict__ xyz, uint32_t n, float *__restrict__ tables) {
    const uint32_t t = blockIdx.x;
    if (t >= n) return;
    const float4 c = xyz[t];
    for (int s = threadIdx.x; s < PSY_SPEC_TABLE; s += blockDim.x)
        tables[(size_t)PSY_SPEC_TABLE * t + s] = s < PSY_MENG_NUM_SAMPLES ? meng_table_value(c.x, c.y, c.z, s) : 0.0f;
}
// For tests: each indexed colour's spectrum at n hero wavelengths, by the
// upsampling and from its table ([colour][i][4] floats each).
__global__ void k_debug_color_spectra(GScene S, const float4 *__restrict__ xyz, uint32_t n_colors,
                                      const float *__restrict__ hero, uint32_t n, float4 *exact, float4 *table) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_colors * n) return;
    const uint32_t t = k / n, i = k % n;
    const float4 c = xyz[t];
    exact[k] = f4(color_to_spectral(GColor{PSY_COLOR_XYZ_K, c.x, c.y, c.z}, hero[i]));
    table[k] = f4(spectrum_from_table(S.spec_tables + (size_t)PSY_SPEC_TABLE * t, hero[i]));
}
cudaError_t launch_debug_color_spectra(const GScene &S, const float4 *d_xyz, uint32_t n_colors, const float *d_hero,
                                       uint32_t n, float *d_exact, float *d_table, cudaStream_t st) {
    const uint32_t total = n_colors * n;
    k_debug_color_spectra<<<(total + 127) / 128, 128, 0, st>>>(S, d_xyz, n_colors, d_hero, n, (float4 *)d_exact,
                                                                  (float4 *)d_table);
    return cudaGetLastError();
}
cudaError_t launch_spectrum_tables(const float4 *d_xyz, uint32_t n, float *d_tables, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_spectrum_tables<<<n, 128, 0, st>>>(d_xyz, n, d_tables);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ accumulate
// XYZ::from_spectral_sample / spp added per pixel (src/renderer.rs:299-310),
// summing the pixel's samples in sample order.
__global__ void k_accumulate(GScene S, const WaveDesc *__restrict__ gwave, PathState P) {
    __shared__ WaveDesc wdesc;
    if (blockIdx.x * blockDim.x >= gwave->npix) return;  // past the wave's pixels, before the copy
    load_wave(gwave, wdesc);
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= wdesc.npix) return;
    const WaveSeg &w = wdesc.seg[seg_of_pixel(wdesc, q)];
    uint32_t lq = q - w.pix_begin;
    uint32_t lr = lq / w.w;
    uint32_t x = w.x0 + (lq - lr * w.w);  // the output row is orow0 + lr
    float inv = (float)w.spp;
    V3 acc = v3(0.0f, 0.0f, 0.0f);
    for (uint32_t s = 0; s < w.spp; s++) {
        uint32_t p = w.path_begin + lq * w.spp + s;
        V3 c = xyz_from_spectral(v4(P.color[p]), P.tw[p].y);
        acc = acc + (c / inv);
    }
    float *o = w.out + ((size_t)(w.orow0 + lr) * w.out_stride + (x - w.out_x0)) * 3;
    o[0] = acc.x; o[1] = acc.y; o[2] = acc.z;
}

cudaError_t launch_accumulate(const GScene &S, const WaveDesc *d_wave, uint32_t max_pix, PathState P, cudaStream_t st) {
    if (max_pix == 0) return cudaSuccess;
    k_accumulate<<<(max_pix + 127) / 128, 128, 0, st>>>(S, d_wave, P);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ sampler values (tests)
// The samplers of the render path evaluated on the device for bit-for-bit
// comparison with the oracle.  args[i] = (a, b, c, d, e); out[i] = 4 words:
//   op 0: hash_u32(a, b)                                   (src/hash.rs:1-10)
//   op 1: hash_u32_to_f32(a, b), f32 bits                  (src/hash.rs:26-29)
//   op 2: golden_ratio_sample(a, b), f32 bits              (src/renderer.rs:728-737)
//   op 3: get_sample_4d(i = a, set = b, px = c, py = d, seed = e), 4 x f32 bits
//                                                          (src/renderer.rs:698-725)
//   op 4: the 4 wavelengths of sample a of pixel (c, d) with seed e, f32 bits
//         (hero from golden_ratio_sample as render_job does, src/renderer.rs:261-265;
//          wavelengths, src/color.rs:20-43)
__global__ void k_debug_samplers(int op, const uint32_t *__restrict__ args, uint32_t n, uint32_t *__restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t *a = args + (size_t)i * 5;
    uint32_t *o = out + (size_t)i * 4;
    float f[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t u0 = 0;
    if (op == 0) {
        u0 = hash_u32(a[0], a[1]);
    } else if (op == 1) {
        u0 = __float_as_uint(hash_u32_to_f32(a[0], a[1]));
    } else if (op == 2) {
        u0 = __float_as_uint(golden_ratio_sample(a[0], a[1]));
    } else if (op == 3) {
        get_sample_4d(a[0], a[1], a[2], a[3], a[4], f);
    } else {
        float hero = map_0_1_to_wavelength(golden_ratio_sample(a[0], hash_u32((a[2] << 16) ^ a[3], a[4])));
        for (int k = 0; k < 4; k++) f[k] = nth_wavelength(hero, k);
    }
    if (op <= 2) {
        o[0] = u0; o[1] = 0u; o[2] = 0u; o[3] = 0u;
    } else {
        for (int k = 0; k < 4; k++) o[k] = __float_as_uint(f[k]);
    }
}
cudaError_t launch_debug_samplers(int op, const uint32_t *d_args, uint32_t n, uint32_t *d_out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_debug_samplers<<<(n + 127) / 128, 128, 0, st>>>(op, d_args, n, d_out);
    return cudaGetLastError();
}

__global__ void k_count_rays(PathState P, uint32_t n, unsigned long long *out) {
    unsigned long long local = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) local += P.flags[i] >> 16;
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, local);
}
cudaError_t launch_count_rays(PathState P, uint32_t n, unsigned long long *out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_count_rays<<<152 * 4, 256, 0, st>>>(P, n, out);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ image output
// Image::write_png's conversion (src/image.rs:138-164, 293-305): XYZ ->
// rec709 (m, row-major, the generated xyz_to_rec709_e), sRGB gamma, clamp
// to [0, 1], x 255 truncated to u8, alpha 255; rows flipped (PNG row 0 is
// the image's last row).
__device__ __forceinline__ float srgb_gamma(float n) {
    return n < 0.0031308f ? n * 12.92f : (1.055f * powf(n, 1.0f / 2.4f)) - 0.055f;
}
__device__ __forceinline__ uint8_t quantize_255(float n) {
    float v = fminf(1.0f, fmaxf(0.0f, n)) * 255.0f;  // NaN -> 0 (Rust's max)
    return (uint8_t)v;
}
__global__ void k_xyz_to_srgb8(const float *__restrict__ xyz, uint32_t w, uint32_t h, Mat3f m,
                               uchar4 *__restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    uint32_t x = i % w, y = i / w;
    const float *p = xyz + ((size_t)(h - 1 - y) * w + x) * 3;
    float X = p[0], Y = p[1], Z = p[2];
    float r = ((X * m.m[0]) + (Y * m.m[1])) + (Z * m.m[2]);
    float g = ((X * m.m[3]) + (Y * m.m[4])) + (Z * m.m[5]);
    float b = ((X * m.m[6]) + (Y * m.m[7])) + (Z * m.m[8]);
    out[i] = make_uchar4(quantize_255(srgb_gamma(r)), quantize_255(srgb_gamma(g)), quantize_255(srgb_gamma(b)), 255);
}
cudaError_t launch_xyz_to_srgb8(const float *xyz, uint32_t w, uint32_t h, const Mat3f &m, uint8_t *rgba,
                                cudaStream_t st) {
    uint32_t n = w * h;
    if (n == 0) return cudaSuccess;
    k_xyz_to_srgb8<<<(n + 255) / 256, 256, 0, st>>>(xyz, w, h, m, reinterpret_cast<uchar4 *>(rgba));
    return cudaGetLastError();
}

// Host helper: set the magenta constant (rec709_to_xyz((1,0,1))) computed by
// the host with the reference's f32 arithmetic.
void psy_set_magenta(const float xyz[3]) {
    GColor c{PSY_COLOR_XYZ_K, xyz[0], xyz[1], xyz[2]};
    cudaMemcpyToSymbol(c_magenta, &c, sizeof(c));
    psy_upload_trace_constants(nullptr, xyz);
    psy_upload_wave_f32_constants(nullptr, xyz);
}
