// The f32 camera and hit-shading kernels of the optimized form (RT = float:
// no FP64 outside the watertight triangle retest).  This translation unit is
// compiled with FMA contraction (--fmad=true): a product feeding a sum rounds
// once, which removes an instruction and a dependent latency from every
// dot product, cross product, lerp and transform of the shading code (the
// kernel's leading stall is waiting on fixed-latency results).  The plain
// form (RT = double, kernels.cu) keeps --fmad=false and rounds every
// operation as the reference's CPU code writes it; the optimized form's
// error against the FP64 oracle is measured, not assumed.  Traversal and
// triangle tests are in trace_kernels.cu (no contraction) in both forms,
// so both forms find the same hits for the same rays.
#include "wave_kernels.cuh"

cudaError_t launch_camera_f32(const GScene &S, const WaveDesc *d_wave, uint32_t max_paths, PathState P, RayBuf R,
                              uint32_t *queue, uint32_t *count, cudaStream_t st) {
    if (max_paths == 0) return cudaSuccess;
    k_camera<float><<<(max_paths + 255) / 256, 256, 0, st>>>(S, d_wave, P, R, queue, count);
    return cudaGetLastError();
}

cudaError_t launch_shade_hit_f32(const GScene &S, const WaveDesc *d_wave, PathState P, RayBuf R, HitBuf H,
                                 const uint32_t *queue, const uint32_t *count, uint32_t max_count,
                                 const QueueOut &out, int minb, int grid, cudaStream_t st) {
#define SH(MB)                                                                                               \
    {                                                                                                        \
        int g = queue_grid((const void *)k_shade_hit<float, MB>, grid, max_count);                           \
        if (g > 0)                                                                                           \
            k_shade_hit<float, MB><<<g, 128, 0, st>>>(S, d_wave, P, R, H, queue, count, out);                 \
    }
    if (minb >= 8) SH(8)
    else if (minb >= 6) SH(6)
    else SH(4)
#undef SH
    return cudaGetLastError();
}

// This unit's copies of the tables the camera and shading read.
void psy_upload_wave_f32_constants(const uint32_t sobol_nib[8][8][16], const float magenta[3]) {
    if (sobol_nib) cudaMemcpyToSymbol(g_sobol_nib, sobol_nib, sizeof(uint32_t) * 8 * 8 * 16);
    if (magenta) {
        GColor c{PSY_COLOR_XYZ_K, magenta[0], magenta[1], magenta[2]};
        cudaMemcpyToSymbol(c_magenta, &c, sizeof(c));
    }
}
