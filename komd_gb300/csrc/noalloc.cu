// noalloc.cu -- ATM forces of a small periodic system without any device
// allocation: komd_gpu_atm_forces_noalloc (include/komd_gpu.h).
//
// Who needs it: callers that hand the engine device pointers but may not
// allocate device memory themselves.  Typical cases are a host application
// whose caching allocator reserved the whole device at start-up (cudaMalloc
// then fails), and a time-step loop that must not call cudaMalloc/cudaFree
// because both implicitly synchronise the device.  Such a caller passes
// positions in and forces out; everything in between lives here.
//
// Scratch: the per-site neighbour list inside cutoff_3b, the per-site counts
// and an overflow flag, in one file-scope __device__ array of fixed size
// (KOMD_NOALLOC_MAX_SITES x KOMD_NOALLOC_NL_CAP entries, about 6.3 MB).  The
// array is device memory of this library's module: CUDA loads modules lazily
// by default (CUDA_MODULE_LOADING=LAZY), so the array is reserved on a device
// when this module is first used there -- by the first call of the entry
// point on that device -- and held until the process exits.  A caller whose
// host application later reserves the rest of the device must therefore make
// its first call (or run with CUDA_MODULE_LOADING=EAGER) before that.
//
// Host code never uses the array's name as an address (on the host it is
// only a stand-in symbol): the first call on each device resolves the device
// address with cudaGetSymbolAddress while that device is current, checks the
// result, caches it, and passes it to the kernels.  That first call on a
// device therefore does this set-up and should come before any stream
// capture on that device.
//
// All calls share the one array and each call overwrites it: the counts are
// rewritten in full and the overflow flag is cleared at the start of every
// call.  Calls whose GPU work overlaps (concurrent streams, or threads
// driving the same device) race on the array and must be serialised by the
// caller.  After KOMD_ERR_OVERFLOW the forces in f are undefined (they come
// from a truncated neighbour list); the next call starts clean.
#include <cstdint>
#include <mutex>
#include <string>

#include "komd_gpu.h"

namespace komd {
void set_last_error(const std::string &msg);   // capi.cu
}

namespace {

constexpr int kMaxSites = KOMD_NOALLOC_MAX_SITES;
constexpr int kCap = KOMD_NOALLOC_NL_CAP;
constexpr int kWarps = 8;
constexpr size_t kListBytes = (size_t)kMaxSites * kCap * sizeof(float4);
constexpr size_t kCountBytes = (size_t)kMaxSites * sizeof(int);
constexpr size_t kScratchBytes = kListBytes + kCountBytes + 256;

// the scratch: neighbour entries (r_i - r_j, unused w), counts, overflow flag
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

struct Box {
    double low[3], L[3];
};

// neighbour list by all pairs with the minimum image (n <= kMaxSites):
// FP64 difference, then the image shift, then FP32 entry
__global__ void k_noalloc_list(int n, const double *__restrict__ r, Box b, double rc2, float4 *__restrict__ nl,
                               int *__restrict__ cnt, int *__restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = r[3 * i], yi = r[3 * i + 1], zi = r[3 * i + 2];
    int c = 0;
    for (int j = 0; j < n; j++) {
        if (j == i) continue;
        double d[3] = {xi - r[3 * j], yi - r[3 * j + 1], zi - r[3 * j + 2]};
        for (int k = 0; k < 3; k++) d[k] -= b.L[k] * rint(d[k] / b.L[k]);
        const double q = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (q > rc2) continue;
        if (c < kCap) nl[(size_t)i * kCap + c] = make_float4((float)d[0], (float)d[1], (float)d[2], 0.f);
        c++;
    }
    cnt[i] = c < kCap ? c : kCap;
    if (c > kCap) atomicOr(flag, 1);
}

// the engine's ATM vertex kernel (FULL triplet set), reading its neighbour
// list from the static scratch and writing (not adding) the ATM force
__global__ void __launch_bounds__(32 * kWarps) k_noalloc_atm(int n, const float4 *__restrict__ nl,
                                                              const int *__restrict__ cnt, float rc2, double scale,
                                                              double *__restrict__ f) {
    __shared__ float4 se[kWarps][kCap];
    __shared__ float2 sq[kWarps][kCap];
    __shared__ unsigned s_q[kWarps][64];
    __shared__ float s_qc[kWarps][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * kWarps + w;
    if (i >= n) return;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const int ni = cnt[i];
    for (int k = lane; k < ni; k += 32) {
        const float4 e = nl[(size_t)i * kCap + k];
        const float A = e.x * e.x + e.y * e.y + e.z * e.z;
        se[w][k] = e;
        sq[w][k] = make_float2(A, 1.0f / A);
    }
    __syncwarp();
    float gx = 0.f, gy = 0.f, gz = 0.f;
    auto triplet = [&](unsigned e, float C) {
        const int a = (int)(e & 0xffffu), b = (int)(e >> 16);
        const float4 ea = se[w][a], eb = se[w][b];
        const float A = sq[w][a].x, B = sq[w][b].x;
        const float s = rsqrtf(A) * rsqrtf(B) * rsqrtf(C);
        const float s2 = s * s, s5 = s2 * s2 * s;
        const float t1 = A + B - C, t2 = A - B + C, t3 = B + C - A;
        const float u = t2 * t3, v = t1 * t3, x = t1 * t2, P = t1 * u;
        const float vA = s5 * (-1.5f * B * C + 0.375f * (u + v - x) - 0.9375f * P * sq[w][a].y);
        const float vB = s5 * (-1.5f * A * C + 0.375f * (u - v + x) - 0.9375f * P * sq[w][b].y);
        gx += vA * ea.x + vB * eb.x;
        gy += vA * ea.y + vB * eb.y;
        gz += vA * ea.z + vB * eb.z;
    };
    int qn = 0;
    const int half = ni / 2;
    for (int a0 = 0; a0 < ni; a0 += 32) {
        const int a = a0 + lane;
        const bool av = a < ni;
        const float4 ea = av ? se[w][a] : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int d = 1; d <= half; d++) {
            bool hit = false;
            int b = 0;
            float C = 0.f;
            if (av && !(2 * d == ni && a >= d)) {
                b = a + d < ni ? a + d : a + d - ni;
                const float4 eb = se[w][b];
                const float cx = eb.x - ea.x, cy = eb.y - ea.y, cz = eb.z - ea.z;
                C = cx * cx + cy * cy + cz * cz;
                hit = C <= rc2;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const int pos = qn + __popc(m & lt);
                s_q[w][pos] = (unsigned)a | ((unsigned)b << 16);
                s_qc[w][pos] = C;
            }
            qn += __popc(m);
            if (qn >= 32) {
                __syncwarp();
                const unsigned e = s_q[w][lane];
                const float ce = s_qc[w][lane];
                const bool mv = lane < qn - 32;
                const unsigned te = mv ? s_q[w][lane + 32] : 0u;
                const float tc = mv ? s_qc[w][lane + 32] : 0.f;
                __syncwarp();
                if (mv) { s_q[w][lane] = te; s_qc[w][lane] = tc; }
                __syncwarp();
                qn -= 32;
                triplet(e, ce);
            }
        }
    }
    __syncwarp();
    if (lane < qn) triplet(s_q[w][lane], s_qc[w][lane]);
    for (int o = 16; o > 0; o >>= 1) {
        gx += __shfl_xor_sync(0xffffffffu, gx, o);
        gy += __shfl_xor_sync(0xffffffffu, gy, o);
        gz += __shfl_xor_sync(0xffffffffu, gz, o);
    }
    if (lane == 0) {
        f[3 * i] = scale * (double)gx;
        f[3 * i + 1] = scale * (double)gy;
        f[3 * i + 2] = scale * (double)gz;
    }
}

int fail(int code, const std::string &m) {
    komd::set_last_error(m);   // reported by komd_gpu_last_error()
    return code;
}

}  // namespace

extern "C" int komd_gpu_atm_forces_noalloc(int64_t n, const double *r, double *f, const double domain_low[3],
                                           const double domain_high[3], double cutoff_3b, double nu,
                                           int32_t atm_sign, void *cuda_stream) {
    if (n <= 0 || !r || !f || !domain_low || !domain_high) return fail(KOMD_ERR_ARG, "bad arguments");
    if (n > kMaxSites)
        return fail(KOMD_ERR_ARG, "komd_gpu_atm_forces_noalloc handles at most " + std::to_string(kMaxSites) +
                                      " sites (its scratch is a fixed static array); got " + std::to_string(n));
    if (!(cutoff_3b > 0)) return fail(KOMD_ERR_ARG, "cutoff_3b must be > 0");
    if (atm_sign != KOMD_ATM_SIGN_REFERENCE && atm_sign != KOMD_ATM_SIGN_PHYSICAL)
        return fail(KOMD_ERR_ARG, "atm_sign must be KOMD_ATM_SIGN_REFERENCE or KOMD_ATM_SIGN_PHYSICAL");
    Box b;
    for (int d = 0; d < 3; d++) {
        b.low[d] = domain_low[d];
        b.L[d] = domain_high[d] - domain_low[d];
        if (!(b.L[d] >= 2.0 * cutoff_3b))
            return fail(KOMD_ERR_ARG, "each box edge must be at least 2 * cutoff_3b (minimum image)");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(KOMD_ERR_ARG, "device index out of range");
    void *base = nullptr;
    {
        // once per device, with that device current: the device address of the scratch
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
            if (e != cudaSuccess || !base)
                return fail(KOMD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_ptr[dev] = base;
        }
        base = g_scratch_ptr[dev];
    }
    float4 *nl = reinterpret_cast<float4 *>(base);
    int *cnt = reinterpret_cast<int *>(static_cast<unsigned char *>(base) + kListBytes);
    int *flag = reinterpret_cast<int *>(static_cast<unsigned char *>(base) + kListBytes + kCountBytes);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    e = cudaMemsetAsync(flag, 0, sizeof(int), st);   // the flag must start at zero on every call
    if (e != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string("clear flag: ") + cudaGetErrorString(e));
    const int ni = (int)n;
    k_noalloc_list<<<(ni + 127) / 128, 128, 0, st>>>(ni, r, b, cutoff_3b * cutoff_3b, nl, cnt, flag);
    const double scale = 2.0 * (atm_sign == KOMD_ATM_SIGN_REFERENCE ? 1.0 : -1.0) * nu;
    k_noalloc_atm<<<(ni + kWarps - 1) / kWarps, 32 * kWarps, 0, st>>>(ni, nl, cnt, (float)(cutoff_3b * cutoff_3b),
                                                                      scale, f);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    int overflow = 0;
    e = cudaMemcpyAsync(&overflow, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(e));
    if (overflow)
        return fail(KOMD_ERR_OVERFLOW, "more than " + std::to_string(kCap) +
                                           " neighbours inside cutoff_3b for a site (fixed scratch capacity)");
    return KOMD_OK;
}
