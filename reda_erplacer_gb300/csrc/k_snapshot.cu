// Headless snapshots of a placement (src/drawing.rs:7-60) and of the density
// map (src/epotential.rs:199-223) into RGB byte buffers, rasterised on the
// device; the caller writes the image file.  No graphics API is involved.
#include "erp_internal.cuh"

namespace erp {

// draw_placement: instance i covers pixels [ceil(x), ceil(x)+ceil(w)) x
// [H - ceil(y) - ceil(h), H - ceil(y)) clipped to the image; later instances
// paint over earlier ones, so a pixel shows the highest index covering it
// (kept with atomicMax, independent of thread order).  Zero-size instances are
// skipped.
__global__ void k_raster_top(int N, const float *__restrict__ x, const float *__restrict__ y,
                             const float *__restrict__ w, const float *__restrict__ h, int W, int H,
                             int *__restrict__ top) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float wc = ceilf(w[i]), hc = ceilf(h[i]);
        if (!(wc >= 1.0f) || !(hc >= 1.0f)) continue;          // w == 0 || h == 0 (or NaN)
        const float xc = ceilf(x[i]), yc = ceilf(y[i]);
        // pixel rectangle, clipped; float bounds first so huge values cannot overflow
        const float fx0 = xc, fy0 = (float)H - yc - hc;
        const float fx1 = fx0 + wc, fy1 = fy0 + hc;
        const int x0 = (int)fmaxf(fx0, 0.0f), x1 = (int)fminf(fx1, (float)W);
        const int y0 = (int)fmaxf(fy0, 0.0f), y1 = (int)fminf(fy1, (float)H);
        for (int py = y0; py < y1; ++py)
            for (int px = x0; px < x1; ++px) atomicMax(top + (size_t)py * W + px, i + 1);
    }
}

// pixel colour: white (no instance), blue (movable), red (fixed)
__global__ void k_raster_rgb(size_t npix, int NM, const int *__restrict__ top, unsigned char *__restrict__ rgb) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        const int t = top[p];
        unsigned char r = 255, g = 255, b = 255;
        if (t > 0) {
            g = 0;
            if (t - 1 >= NM) { r = 255; b = 0; }
            else { r = 0; b = 255; }
        }
        rgb[3 * p] = r;
        rgb[3 * p + 1] = g;
        rgb[3 * p + 2] = b;
    }
}

// min and max of the map (exact in any order)
__global__ void k_map_minmax(size_t mn, const float *__restrict__ map, unsigned *__restrict__ out) {
    float lo = INFINITY, hi = -INFINITY;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < mn; k += (size_t)gridDim.x * blockDim.x) {
        lo = fminf(lo, map[k]);
        hi = fmaxf(hi, map[k]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    // order-preserving unsigned keys of the floats
    auto key = [](float v) {
        const unsigned u = __float_as_uint(v);
        return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    };
    if ((threadIdx.x & 31) == 0) {
        atomicMin(out, key(lo));
        atomicMax(out + 1, key(hi));
    }
}

__device__ __forceinline__ float unkey(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// draw_density_map: normalised = clamp((v - min) / (max - min + 1e-12), 0, 1);
// (r, g, b) = (normalised * 255, 0, (1 - normalised) * 255) truncated; bin
// (i, j) goes to pixel column i, row n - 1 - j (image m wide, n high).
__global__ void k_density_rgb(int m, int n, const float *__restrict__ map, const unsigned *__restrict__ mm,
                              unsigned char *__restrict__ rgb) {
    const float lo = unkey(mm[0]), hi = unkey(mm[1]);
    const float den = __fadd_rn(__fsub_rn(hi, lo), 1e-12f);
    const size_t mn = (size_t)m * n;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < mn; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / n), j = (int)(idx - (size_t)i * n);
        float v = __fdiv_rn(__fsub_rn(map[idx], lo), den);
        v = fminf(fmaxf(v, 0.0f), 1.0f);
        const size_t p = (size_t)(n - 1 - j) * m + i;
        rgb[3 * p] = (unsigned char)__fmul_rn(v, 255.0f);
        rgb[3 * p + 1] = 0;
        rgb[3 * p + 2] = (unsigned char)__fmul_rn(__fsub_rn(1.0f, v), 255.0f);
    }
}

static int grid_of(size_t work) {
    size_t g = (work + kThreads - 1) / kThreads;
    return (int)(g < 1 ? 1 : (g > 152 * 8 ? 152 * 8 : g));
}

cudaError_t launch_snapshot_placement(Ctx &c, int W, int H, unsigned char *d_rgb, int *d_top) {
    const size_t npix = (size_t)W * H;
    cudaError_t e = cudaMemsetAsync(d_top, 0, sizeof(int) * npix, c.stream);
    if (e != cudaSuccess) return e;
    if (c.N > 0) k_raster_top<<<grid_of(c.N), kThreads, 0, c.stream>>>(c.N, c.x, c.y, c.w, c.h, W, H, d_top);
    k_raster_rgb<<<grid_of(npix), kThreads, 0, c.stream>>>(npix, c.NM, d_top, d_rgb);
    return cudaGetLastError();
}

cudaError_t launch_snapshot_density(Ctx &c, const float *map, unsigned char *d_rgb, unsigned *d_mm) {
    const unsigned init[2] = {0xffffffffu, 0u};
    cudaError_t e = cudaMemcpyAsync(d_mm, init, sizeof init, cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return e;
    const size_t mn = (size_t)c.m * c.n;
    k_map_minmax<<<grid_of(mn), kThreads, 0, c.stream>>>(mn, map, d_mm);
    k_density_rgb<<<grid_of(mn), kThreads, 0, c.stream>>>(c.m, c.n, map, d_mm, d_rgb);
    return cudaGetLastError();
}

}  // namespace erp
