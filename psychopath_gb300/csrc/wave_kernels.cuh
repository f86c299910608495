// Wave kernels shared by two translation units: the camera and hit-shading
// kernels are templates on the shading arithmetic RT.  kernels.cu
// instantiates RT = double (the reference's precision, every operation
// rounded as written: the plain form) and wave_f32.cu RT = float (the
// optimized form, compiled with FMA contraction).
#pragma once

#include "dev_bins.cuh"
#include "dev_surface.cuh"
#include "kernels.cuh"

using namespace psyd;

// ------------------------------------------------------------------ wave segments
// Copies the wave descriptor into shared memory (one read per block).
__device__ __forceinline__ void load_wave(const WaveDesc *__restrict__ g, WaveDesc &sm) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g);
    uint32_t *dst = reinterpret_cast<uint32_t *>(&sm);
    for (int i = threadIdx.x; i < (int)(sizeof(WaveDesc) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
}
__device__ __forceinline__ int seg_of_path(const WaveDesc &wd, uint32_t p) {
    int i = 0;
    while (i + 1 < (int)wd.nseg && p >= wd.seg[i + 1].path_begin) i++;
    return i;
}
__device__ __forceinline__ int seg_of_pixel(const WaveDesc &wd, uint32_t q) {
    int i = 0;
    while (i + 1 < (int)wd.nseg && q >= wd.seg[i + 1].pix_begin) i++;
    return i;
}

// ------------------------------------------------------------------ camera
// Ray generation of Renderer::render_job (src/renderer.rs:241-275) and
// LightPath::new (src/renderer.rs:392-431) / Camera::generate_ray
// (src/camera.rs:74-102).
template <class RT>
__global__ void k_camera(GScene S, const WaveDesc *__restrict__ gwave, PathState P, RayBuf R, uint32_t *queue,
                         uint32_t *count) {
    __shared__ WaveDesc wdesc;
    // blocks past the wave's paths (the grid covers its capacity) leave
    // before the descriptor copy; block 0 always stays to write the count
    if (blockIdx.x > 0 && blockIdx.x * blockDim.x >= gwave->npaths) return;
    load_wave(gwave, wdesc);
    uint32_t n = wdesc.npaths;
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *count = n;
    if (p >= n) return;
    const WaveSeg &w = wdesc.seg[seg_of_path(wdesc, p)];
    uint32_t lp = (p - w.path_begin) / w.spp, si = (p - w.path_begin) - lp * w.spp;
    uint32_t x = w.x0 + lp % w.w, y = w.y0 + (lp / w.w) * w.ystep;
    float cmpx = 1.0f / (float)w.img_w, cmpy = 1.0f / (float)w.img_h;
    float min_x = -1.0f, max_x = 1.0f;
    float min_y = -((float)w.img_h / (float)w.img_w), max_y = (float)w.img_h / (float)w.img_w;
    float xe = max_x - min_x, ye = max_y - min_y;
    float d[4], d4[4];
    get_sample_4d(si, 0, x, y, w.seed, d);
    get_sample_4d(si, 1, x, y, w.seed, d4);
    float fx = probit<RT>(d[3], 2.0f / 6.0f) + 0.5f;
    float fy = probit<RT>(d4[0], 2.0f / 6.0f) + 0.5f;
    float sx = (fx + (float)x) * cmpx;
    float sy = (fy + (float)y) * cmpy;
    float ix = (sx - 0.5f) * xe, iy = (0.5f - sy) * ye;
    float wl = map_0_1_to_wavelength(golden_ratio_sample(si, hash_u32((x << 16) ^ y, w.seed)));
    float time = d[0];
    // Camera::generate_ray
    Xf xf = lerp_slice_xf(S.cam_xf, S.n_cam_xf, time);
    float tfov = lerp_slice_f(S.cam_tfov, S.n_cam_tfov, time);
    float ar = lerp_slice_f(S.cam_ap, S.n_cam_ap, time);
    float fd = lerp_slice_f(S.cam_fd, S.n_cam_fd, time);
    float cu, cv;
    square_to_circle((d[1] * 2.0f) - 1.0f, (d[2] * 2.0f) - 1.0f, &cu, &cv);
    V3 orig = v3(ar * cu, ar * cv, 0.0f);
    V3 dir = normalized(v3((ix * tfov) - (orig.x / fd), (iy * tfov) - (orig.y / fd), 1.0f));
    V3 wo = xf_point(orig, xf), wd = xf_vector(dir, xf);
    // The path's colour starts at 0 (the pixel sum reads it whatever the
    // path does).  Its light attenuation (1), closure-sample pdf (1),
    // pending light, next attenuation and next bounce ray are not stored:
    // k_shade_hit takes the first two as constants for a camera event and
    // writes the others before anything reads them.
    P.color[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.tw[p] = make_float2(time, wl);
    P.seed[p] = w.seed ^ 0x40d4682bu;
    P.flags[p] = 0u;  // EV_CAMERA, bounce 0, no next bounce, 0 rays
    R.o[p] = make_float4(wo.x, wo.y, wo.z, CUDART_INF_F);
    R.d[p] = make_float4(wd.x, wd.y, wd.z, time);
    R.occl[p] = 0;
    queue[p] = p;
}

// ------------------------------------------------------------------ shade
#define EV_CAMERA 0u
#define EV_BOUNCE 1u
#define EV_SHADOW 2u

// Appends the live paths of the warp to out.queue (one atomic per warp),
// with their sort keys when out.keys is set.
__device__ __forceinline__ void push_live(bool alive, uint32_t p, uint32_t key, const QueueOut &out) {
    unsigned mask = __ballot_sync(__activemask(), alive);
    if (mask == 0) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(out.count, (uint32_t)__popc(mask));
    base = __shfl_sync(__activemask(), base, leader);
    if (alive) {
        uint32_t i = base + __popc(mask & ((1u << lane) - 1u));
        out.queue[i] = p;
        if (out.keys) out.keys[i] = key;
    }
}
// The sort key of a path's next ray (two-point key, occlusion flag above).
__device__ __forceinline__ uint32_t next_ray_key(const QueueOut &out, V3 o, V3 d, bool occl) {
    return two_point_key(o.x, o.y, o.z, d.x, d.y, d.z, out.lo, out.inv, out.len, out.p) |
           ((occl ? 1u : 0u) << (6 * out.p));
}

// LightPath::next (src/renderer.rs:449-691), in two kernels over the same
// queue of paths whose rays were just traced: k_shade_hit takes the paths
// whose ray was a camera or bounce ray (surface hit, emission, background,
// light sample and bounce -- the heavy part), k_shade_shadow those whose ray
// was a shadow ray (add the pending light, set up the next bounce -- a few
// loads and stores).  Each skips the other kind, so the shadow results run
// at the occupancy of their own small register footprint rather than the
// hit kernel's; a queue ordered by ray key (the occlusion flag is its top
// bit) keeps the kinds contiguous, so skipped warps leave at once.
// k_shade_shadow runs first and marks the paths it shaded (PSY_SHADED_BIT
// in their flags); k_shade_hit skips the marked paths and clears the mark,
// so each path of the queue is shaded once per iteration.
#define PSY_SHADED_BIT (1u << 11)
template <class RT, int MINB>
__global__ void __launch_bounds__(128, MINB) k_shade_hit(GScene S, const WaveDesc *__restrict__ gwave, PathState P,
                                                   RayBuf R, HitBuf H, const uint32_t *__restrict__ queue,
                                                   const uint32_t *__restrict__ count, QueueOut out) {
    __shared__ WaveDesc wdesc;
    uint32_t n = *count;
    // blocks past the queue's length (the grid covers the wave's capacity)
    // leave at once, before the descriptor copy and its barrier
    if (blockIdx.x * blockDim.x >= n) return;
    load_wave(gwave, wdesc);
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
        if (q < n && (fl & PSY_SHADED_BIT)) {
            P.flags[p] = fl & ~PSY_SHADED_BIT;  // shaded by k_shade_shadow this iteration
        } else if (q < n) {
            uint32_t ev = fl & 3u, bounce = (fl >> 2) & 0xFFu, has_nb = (fl >> 10) & 1u, nrays = fl >> 16;
            nrays += 1;
            float2 tw = P.tw[p];
            float time = tw.x, wl = tw.y;
            uint4 ki = H.ki[p];
            // colour, light attenuation and closure-sample pdf: a camera
            // event's are the path's initial 0, 1 and 1 (k_camera stores the
            // colour only)
            const bool cam = ev == EV_CAMERA;
            V4 color = cam ? splat4(0.0f) : v4(P.color[p]);
            V4 latt = cam ? splat4(1.0f) : v4(P.latt[p]);
            float csp = cam ? 1.0f : P.nb_o[p].w;
            // the hit's barycentrics, the ray and the sampling state
            float4 tb = H.tb[p];
            float4 ro = R.o[p], rd = R.d[p];
            V3 o = v3(ro), d = v3(rd);
            uint32_t seed = P.seed[p];
            const WaveSeg &w = wdesc.seg[seg_of_path(wdesc, p)];
            uint32_t lp = p - w.path_begin;
            uint32_t pix = lp / w.spp;
            uint32_t si = lp - pix * w.spp;
            uint32_t px = w.x0 + pix % w.w, py = w.y0 + (pix / w.w) * w.ystep;
            if (ki.x == PSY_HIT_SURFACE_K || ki.x == PSY_HIT_LIGHT_K) {
                HitRec h;
                h.kind = ki.x; h.prim = ki.y; h.slot = ki.z;
                h.t = tb.x; h.b0 = tb.y; h.b1 = tb.z; h.b2 = tb.w;
                SurfData sd;
                resolve_hit<RT>(S, h, o, d, time, sd);
                const Closure &cl = sd.closure;
                if (cl.kind == PSY_CL_EMIT) {
                    V4 c = color_spectrum<RT>(S, cl.color, wl);
                    if (ev == EV_CAMERA) {
                        color = color + c;
                    } else {
                        float mis = power_heuristic(csp, sd.sample_pdf);
                        color = color + c * latt / splat4(mis);
                    }
                    P.color[p] = f4(color);
                } else {
                    latt = latt / splat4(csp);
                    seed += 1;
                    // the surface colour's spectrum: shared by the light
                    // sample's evaluation and the bounce sample
                    V4 cspec = color_spectrum<RT>(S, cl.color, wl);
                    float smp[4];
                    get_sample_4d(si, 0, px, py, seed, smp);
                    LightSample li = scene_sample_lights<RT>(S, smp[0], smp[1], smp[2], wl, time, d, sd.pos,
                                                             sd.nor, sd.nor_g, cl);
                    bool found = false;
                    if (li.kind != 0 && !(li.pdf <= 0.0f) && !(li.sel_pdf <= 0.0f)) {
                        // the direction to the light (a distant light's own,
                        // else toward the sampled point); the evaluation and
                        // the shadow ray's origin run once for both kinds, so
                        // a warp whose lanes sampled different kinds does
                        // not run them twice
                        V3 ldir = li.kind == 1 ? li.dir : li.sp - sd.pos;
                        float cpdf;
                        V4 att = closure_evaluate(cl, cspec, d, ldir, sd.nor, sd.nor_g, &cpdf);
                        V3 so = robust_ray_origin(sd.pos, sd.pos_err, normalized(sd.nor_g), ldir);
                        V3 sdir = ldir;
                        float smax = CUDART_INF_F;
                        if (li.kind != 1) {
                            V3 oe = robust_ray_origin(li.sp, li.serr, normalized(li.sn), neg(ldir));
                            sdir = oe - so;
                            smax = 1.0f;
                        }
                        if (!(max_elem4(att) <= 0.0f)) {
                            float lmis = power_heuristic(li.pdf, cpdf);
                            V4 pend = li.color * att * latt / splat4(lmis * li.sel_pdf);
                            P.pending[p] = f4(pend);
                            R.o[p] = make_float4(so.x, so.y, so.z, smax);
                            R.d[p] = make_float4(sdir.x, sdir.y, sdir.z, time);
                            R.occl[p] = 1;
                            found = true;
                            if (out.keys) key = next_ray_key(out, so, sdir, true);
                        }
                    }
                    bool do_bounce = false;
                    V4 nafac = splat4(1.0f);  // set with a bounce that succeeds
                    V3 nbo = v3(0.0f, 0.0f, 0.0f), nbd = v3(0.0f, 0.0f, 0.0f);  // the bounce ray
                    if (bounce < S.max_bounces) {
                        bounce += 1;
                        seed += 1;
                        float b4[4];
                        get_sample_4d(si, 0, px, py, seed, b4);
                        V3 dir;
                        float pdf;
                        V4 filt = closure_sample(cl, cspec, d, sd.nor, sd.nor_g, b4[0], b4[1], &dir, &pdf);
                        if ((pdf > 0.0f) && (max_elem4(filt) > 0.0f)) {
                            nafac = filt;
                            csp = pdf;
                            nbo = robust_ray_origin(sd.pos, sd.pos_err, normalized(sd.nor_g), dir);
                            nbd = dir;
                            P.nafac[p] = f4(nafac);
                            P.nb_o[p] = make_float4(nbo.x, nbo.y, nbo.z, csp);
                            P.nb_d[p] = make_float4(nbd.x, nbd.y, nbd.z, 0.0f);
                            has_nb = 1;
                            do_bounce = true;
                        }
                    } else {
                        has_nb = 0;
                    }
                    // the stored attenuation is the bounce ray's (the light
                    // sample's pending light above used the current one):
                    // k_shade_shadow sets up a stored bounce with it as is.
                    // A bounce sample that fails keeps the path's earlier
                    // bounce ray and factor (as the reference's LightPath
                    // does): with a shadow ray, that stale bounce is set up
                    // after it, times the stored factor
                    if (do_bounce) latt = latt * nafac;
                    else if (found && has_nb) latt = latt * v4(P.nafac[p]);
                    if (found) {
                        ev = EV_SHADOW;
                        alive = true;
                    } else if (do_bounce) {
                        R.o[p] = make_float4(nbo.x, nbo.y, nbo.z, CUDART_INF_F);
                        R.d[p] = make_float4(nbd.x, nbd.y, nbd.z, time);
                        R.occl[p] = 0;
                        ev = EV_BOUNCE;
                        alive = true;
                        if (out.keys) key = next_ray_key(out, nbo, nbd, false);
                    }
                    P.latt[p] = f4(latt);
                    P.seed[p] = seed;
                }
            } else {
                V4 bg = color_spectrum<RT>(S, S.background, wl);
                color = color + bg * latt / splat4(csp);
                P.color[p] = f4(color);
            }
            P.flags[p] = ev | (bounce << 2) | (has_nb << 10) | (nrays << 16);
        }
        push_live(alive, p, key, out);
    }
}
