// oz_noalloc.cu -- the Ozaki DGEMM on device arrays with no device allocation.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or caching allocator (which must see every byte it
// hands out and may not be bypassed), code that must not trigger the implicit
// device synchronisation of cudaMalloc/cudaFree (latency-critical serving
// paths), and code in environments whose memory budget is fixed before the
// library is called.  For them ozgb_dgemm_device_noalloc takes all of its
// scratch (row/column exponents, the int8-valued slice planes, the device error
// word) from one file-scope __device__ array of kNoAllocScratchBytes, which the
// CUDA runtime reserves once per device when the module loads.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and checks that the device is
// an sm_103 part; later calls on that device reuse the address.  That first call
// should come before any stream capture.
//
// Every call on a device shares the one array and leaves its contents behind;
// each call clears what must start at zero (the column exponents and the error
// word).  Calls whose executions overlap on the GPU (other streams, other host
// threads) race on the array and corrupt each other's results.
//
// The status covers argument checks and launches only: the call returns before
// the kernels run.  A device-side wait that runs out of time (the GEMM stops
// early and leaves C incomplete) is recorded in the array's error word, which
// this entry point does not read back and the next call clears.  A caller that
// must detect that case uses ozgb_dgemm_device and ozgb_sync instead.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "oz_gb300.h"
#include "oz_internal.h"
#include "oz_plan.h"

namespace ozgb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
unsigned char *g_base[kMaxDevices] = {nullptr};

size_t round256(size_t n) { return (n + 255) & ~size_t(255); }

// Device address of the scratch array on the current device (set up once).
ozgb_status scratch_base(unsigned char **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return OZGB_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        int major = 0, minor = 0;
        if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) {
            cudaGetLastError();
            return OZGB_ERR_NO_DEVICE;
        }
        if (major != 10 || minor != 3) return OZGB_ERR_IMAGE;
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return OZGB_ERR_EXEC;
        }
        g_base[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_base[dev];
    return OZGB_OK;
}

}  // namespace
}  // namespace ozgb

using namespace ozgb;

extern "C" ozgb_status ozgb_dgemm_device_noalloc(int M, int N, int K, const double *dA, long lda, const double *dB,
                                                 long ldb, double *dC, long ldc, int slices, void *stream) {
    if (M < 1 || N < 1 || K < 1) return OZGB_ERR_DIMS;
    if (!dA || !dB || !dC || lda < K || ldb < N || ldc < N || slices < 2 || slices > 16) return OZGB_ERR_ARG;
    OzConfig cfg;
    cfg.b = 7;
    cfg.s = slices;
    cfg.J = slices;
    cfg.rounding = OUT_RN;
    Plan p;
    std::string why;
    if (!make_plan(M, N, K, cfg, &p, &why)) return OZGB_ERR_UNSUPPORTED;

    // scratch layout: [error word][er: M][ec: N][A slice blocks][B slice blocks]
    const size_t off_er = 256;
    const size_t off_ec = off_er + round256(sizeof(int32_t) * M);
    const size_t off_at = off_ec + round256(sizeof(int32_t) * N);
    const size_t off_bt = off_at + round256(p.a_bytes);
    const size_t need = off_bt + round256(p.b_bytes);
    if (need > kNoAllocScratchBytes) return OZGB_ERR_TOO_LARGE;

    // an error left pending by earlier, unrelated work on this thread is cleared
    // here, so that the checks below report only what this call launched
    cudaGetLastError();
    unsigned char *base = nullptr;
    const ozgb_status rc = scratch_base(&base);
    if (rc != OZGB_OK) return rc;
    int *err = reinterpret_cast<int *>(base);
    int32_t *er = reinterpret_cast<int32_t *>(base + off_er);
    int32_t *ec = reinterpret_cast<int32_t *>(base + off_ec);
    uint16_t *at = reinterpret_cast<uint16_t *>(base + off_at);
    uint16_t *bt = reinterpret_cast<uint16_t *>(base + off_bt);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // the previous call's contents stay in the array: zero what is accumulated into
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess ||
        cudaMemsetAsync(ec, 0, sizeof(int32_t) * N, st) != cudaSuccess) {
        cudaGetLastError();
        return OZGB_ERR_EXEC;
    }
    launch_rowmax(dA, lda, M, K, er, nullptr, st);
    launch_colmax(dB, ldb, K, N, ec, nullptr, st);
    launch_split_a(dA, lda, M, K, er, p.cfg.b, p.cfg.s, p.KC, p.n_kc, p.Mp, at, st, false, p.f8);
    launch_split_b(dB, ldb, K, N, ec, p.cfg.b, p.cfg.s, p.KC, p.n_kc, p.BN, p.Np, bt, st, false, p.f8);
    if (cudaGetLastError() != cudaSuccess) return OZGB_ERR_EXEC;  // a stage (a) or (b) launch

    GemmArgs g;
    std::memset(&g, 0, sizeof g);
    g.a_tiles = at;
    g.b_tiles = bt;
    g.er = er;
    g.ec = ec;
    g.c = dC;
    g.ldc = ldc;
    g.M = M;
    g.N = N;
    g.n_kc = p.n_kc;
    g.KC = p.KC;
    g.s = p.cfg.s;
    g.J = p.cfg.J;
    g.b = p.cfg.b;
    g.out_mode = OUT_RN;
    g.tiles_m = p.tiles_m;
    g.tiles_n = p.tiles_n;
    g.total_tiles = p.tiles_m * p.tiles_n;
    g.alpha = 1.0;  // C = A B
    g.beta = 0.0;
    g.stages = p.stages;
    g.stage_bytes = p.stage_bytes;
    g.a_block_bytes = p.a_block_bytes;
    g.b_block_bytes = p.b_block_bytes;
    g.b_pad_lo_bytes = static_cast<uint32_t>(p.pad_lo) * p.b_slice_bytes;
    g.b_region_bytes = p.b_region_bytes;
    g.tmem_cols = p.tmem_cols;
    g.err = err;
    g.timeout_ns = 2000000000ull;
    g.n_acc = p.n_acc;
    g.n_iss = p.n_iss;
    for (int a = 0; a < kMaxAcc; ++a) g.acc_t0[a] = p.acc_t0[a];
    g.G = p.G;
    for (int i = 0; i < p.G; ++i) {
        g.blk_lo[i] = p.blk_lo[i];
        g.blk_nb[i] = p.blk_nb[i];
        g.blk_p0[i] = p.blk_p0[i];
        g.blk_p1[i] = p.blk_p1[i];
        g.blk_period[i] = p.blk_period[i];
        g.blk_off[i] = p.blk_off[i];
        g.blk_col1[i] = p.blk_col1[i];
    }
    g.dbl_mask = p.dbl_mask;
    p.fn(g, p.tiles_m * p.tiles_n, p.smem, st);
    if (cudaGetLastError() != cudaSuccess) return OZGB_ERR_EXEC;  // the slice-pair GEMM launch
    return OZGB_OK;
}
