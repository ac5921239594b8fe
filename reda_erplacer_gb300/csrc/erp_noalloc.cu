// Allocation-free spectral Poisson solve (erp_spectral_solve_noalloc).
//
// Some callers of this library cannot call cudaMalloc/cudaFree: a host whose
// device memory is owned by another allocator (a framework's caching allocator
// or a pool that reserves the GPU's memory at start-up, where a library's own
// cudaMalloc can fail or fragment that pool), and placement loops that must not
// stall, since cudaFree synchronises the whole device.  This entry point runs the
// same three spectral passes as erp_spectral_solve, but every intermediate lives
// in the file-scope device array below instead of memory it allocates.
//
// Limits and sharing rules:
//  * at most kMaxBins = 512 x 512 bins (the reference's fixed grid,
//    src/placement.rs:50); larger grids are rejected with ERP_EINVAL;
//  * the array (about 4.1 MiB) is held by every GPU that loads the library,
//    until the process exits;
//  * every call shares the array: each call rewrites all of it that it reads
//    (twiddle tables, the state words, the intermediates), so consecutive calls
//    are independent, but calls that overlap on the GPU (two streams, or two
//    host threads) race with each other;
//  * the first call on a device does that device's set-up (it looks up the
//    array's device address with cudaGetSymbolAddress and sets the kernels'
//    shared-memory limits); make that first call before any stream capture.
//    The address is kept for the life of the process, so cudaDeviceReset on a
//    device after its first call is not supported (the reset rebuilds the
//    module and moves the array);
//  * the twiddle tables are built on the device here, and on the host for
//    erp_spectral_solve, so the two solves agree within FP32 rounding (the
//    tests' 1e-5 relative L2), not bit for bit.
#include <math.h>

#include <mutex>
#include <string>

#include "erp_internal.cuh"

namespace erp {

namespace {

constexpr size_t kMaxBins = ERP_NOALLOC_MAX_BINS;
constexpr int kMaxSide = 4096;
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kMapBytes = align256(sizeof(float) * kMaxBins);
constexpr size_t kOffT1 = 0;
constexpr size_t kOffTx = kOffT1 + kMapBytes;
constexpr size_t kOffTy = kOffTx + kMapBytes;
constexpr size_t kOffTp = kOffTy + kMapBytes;
constexpr size_t kOffTwM = kOffTp + kMapBytes;
constexpr size_t kOffTwN = kOffTwM + align256(sizeof(float2) * (kMaxSide / 2));
constexpr size_t kOffEkM = kOffTwN + align256(sizeof(float2) * (kMaxSide / 2));
constexpr size_t kOffEkN = kOffEkM + align256(sizeof(float2) * kMaxSide);
constexpr size_t kOffWu = kOffEkN + align256(sizeof(float2) * kMaxSide);
constexpr size_t kOffWv = kOffWu + align256(sizeof(float) * kMaxSide);
constexpr size_t kOffState = kOffWv + align256(sizeof(float) * kMaxSide);
constexpr size_t kScratchBytes = kOffState + align256(sizeof(DevState));

// The scratch.  Host code must not pass this name to a kernel: on the host it is
// a stand-in object, not a device address; the address comes from
// cudaGetSymbolAddress at set-up.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
void *g_scratch_dev[kMaxDevices];
bool g_ready[kMaxDevices];

// Twiddle / frequency tables of one (m, n, bin size) and a cleared state block.
// The trigonometric tables use FP64 sincospi; the frequency vectors repeat the
// FP32 operations of src/frequencies.rs:10-21.
__global__ void k_noalloc_tables(int m, int n, float bin_w, float bin_h, float2 *tw_m, float2 *tw_n,
                                 float2 *ek_m, float2 *ek_n, float *wu, float *wv, DevState *st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double s, c;
    if (t < m / 2) { sincospi(-2.0 * t / m, &s, &c); tw_m[t] = make_float2((float)c, (float)s); }
    if (t < n / 2) { sincospi(-2.0 * t / n, &s, &c); tw_n[t] = make_float2((float)c, (float)s); }
    if (t < m) {
        sincospi((double)t / (2.0 * m), &s, &c);
        ek_m[t] = make_float2((float)c, (float)-s);
        const float tpm = __fdiv_rn((float)(2.0 * 3.14159265358979323846), (float)m);
        wu[t] = __fmul_rn((float)t, tpm);
    }
    if (t < n) {
        sincospi((double)t / (2.0 * n), &s, &c);
        ek_n[t] = make_float2((float)c, (float)-s);
        const float tpn = __fdiv_rn((float)(2.0 * 3.14159265358979323846), (float)n);
        wv[t] = __fmul_rn(__fmul_rn((float)t, tpn), __fdiv_rn(bin_w, bin_h));
    }
    if (t < (int)(sizeof(DevState) / sizeof(int))) reinterpret_cast<int *>(st)[t] = 0;
}

bool pow2_side(int v) { return v >= 16 && v <= kMaxSide && (v & (v - 1)) == 0; }

erp_status device_setup(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_thread_error("no CUDA device available");
        return ERP_ENODEV;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_thread_error("device ordinal beyond the allocation-free solve's table");
        return ERP_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_ready[dev]) {
        int major = 0, minor = 0;
        if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) {
            cudaGetLastError();
            set_thread_error("cannot query the current device");
            return ERP_ENODEV;
        }
        if (major != 10 || minor != 3) {
            set_thread_error("the current device is not sm_103; this library is built for sm_103a only");
            return ERP_ENODEV;
        }
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_thread_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return ERP_ECUDA;
        }
        e = spectral_prepare();
        if (e != cudaSuccess) {
            set_thread_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return ERP_ECUDA;
        }
        g_scratch_dev[dev] = p;
        g_ready[dev] = true;
    }
    *out = g_scratch_dev[dev];
    return ERP_OK;
}

}  // namespace
}  // namespace erp

using namespace erp;

extern "C" erp_status erp_spectral_solve_noalloc(int32_t m, int32_t n, float bin_w, float bin_h,
                                                 const float *rho, float *field_x, float *field_y,
                                                 float *potential, void *stream) {
    if (!pow2_side(m) || !pow2_side(n)) {
        set_thread_error("bin counts must be powers of two in [16, 4096]");
        return ERP_EINVAL;
    }
    if ((size_t)m * (size_t)n > kMaxBins) {
        set_thread_error("the allocation-free spectral solve supports at most 512 x 512 = 262144 bins");
        return ERP_EINVAL;
    }
    if (!rho || !field_x || !field_y || !(bin_w > 0) || !(bin_h > 0)) {
        set_thread_error("invalid spectral solve arguments");
        return ERP_EINVAL;
    }
    void *base = nullptr;
    erp_status s = device_setup(&base);
    if (s != ERP_OK) return s;
    unsigned char *b = static_cast<unsigned char *>(base);
    SpectralPlan p;
    p.m = m; p.n = n; p.logm = ilog2(m); p.logn = ilog2(n);
    p.bin_w = bin_w; p.bin_h = bin_h;
    p.t1 = reinterpret_cast<float *>(b + kOffT1);
    p.tx = reinterpret_cast<float *>(b + kOffTx);
    p.ty = reinterpret_cast<float *>(b + kOffTy);
    p.tp = reinterpret_cast<float *>(b + kOffTp);
    p.tw_m = reinterpret_cast<float2 *>(b + kOffTwM);
    p.tw_n = reinterpret_cast<float2 *>(b + kOffTwN);
    p.ek_m = reinterpret_cast<float2 *>(b + kOffEkM);
    p.ek_n = reinterpret_cast<float2 *>(b + kOffEkN);
    p.wu = reinterpret_cast<float *>(b + kOffWu);
    p.wv = reinterpret_cast<float *>(b + kOffWv);
    p.st = reinterpret_cast<DevState *>(b + kOffState);
    p.partials = nullptr;
    p.stream = static_cast<cudaStream_t>(stream);
    const int side = m > n ? m : n;
    k_noalloc_tables<<<(side + kThreads - 1) / kThreads, kThreads, 0, p.stream>>>(
        m, n, bin_w, bin_h, p.tw_m, p.tw_n, p.ek_m, p.ek_n, p.wu, p.wv, p.st);
    SpectralArgs a;
    a.rho_in = rho;
    a.fx = field_x;
    a.fy = field_y;
    a.psi = potential;
    a.st = p.st;
    launch_spectral_plan(p, a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_thread_error(std::string("spectral solve launch: ") + cudaGetErrorString(e));
        return ERP_ECUDA;
    }
    return ERP_OK;
}
