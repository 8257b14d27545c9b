// Cost of back-to-back tcgen05.mma instructions (cta_group::1) on this GPU, as
// the planner models it: one CTA per SM, one thread issues `n` UMMAs of a given
// M, N and kind into R accumulator ranges used round-robin, with operands that
// change from one instruction to the next; SM cycles per instruction are
// measured with clock64 between the first issue and the commit's arrival.
//
// Prints one line per configuration:  kind M N R cycles_per_umma flop_per_cycle_per_sm
// Every wait on the commit's mbarrier is bounded (1 s); a timeout prints TIMEOUT
// and the program exits 3 after releasing TMEM.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../ozaie_gb300/csrc/oz_ptx.cuh"

using namespace ozgb;

namespace {

constexpr int kASlices = 8;
constexpr int kABytes = 4096;      // 128 rows x 32 bytes (one K step)
constexpr int kBBytes = 256 * 32;  // 256 rows x 32 bytes
constexpr int kBCopies = 4;
constexpr int kSmem = 120 * 1024;  // more than half of the SM: one CTA per SM (TMEM 512 columns)

struct Cfg {
    int M, N, R, f8, n_instr;
};

__global__ void __launch_bounds__(128, 1) umma_cost(const Cfg c, unsigned long long *cycles, int *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *Ab = smem;
    uint8_t *Bb = smem + kASlices * kABytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(Bb + kBCopies * kBBytes);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    for (int i = threadIdx.x * 16; i < kASlices * kABytes + kBCopies * kBBytes; i += blockDim.x * 16)
        *reinterpret_cast<uint4 *>(smem + i) = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    const int warp = threadIdx.x >> 5;
    if (warp == 0) {
        tmem_alloc(slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (threadIdx.x == 32) {
        const uint64_t a0 = smem_desc(smem_u32(Ab), 128, 256);
        const uint64_t b0 = smem_desc(smem_u32(Bb), 128, 256);
        const uint32_t id = c.f8 ? idesc_e4m3_f32(c.M, c.N) : idesc_bf16_f32(c.M, c.N);
        const int dstride = c.R == 1 ? 0 : 512 / c.R;
        const int zero = 0;
        bool ok = true;
        long long t0 = 0;
        for (int pass = 0; pass < 2 && ok; ++pass) {  // pass 0 warms up
            if (pass == 1) t0 = clock64();
            int r = 0, ai = 0, bi = 0;
            for (int i = 0; i < c.n_instr; ++i) {
                const uint32_t d = tmem + static_cast<uint32_t>(r * dstride);
                const uint64_t ad = a0 + static_cast<uint64_t>(ai) * (kABytes >> 4);
                const uint64_t bd = b0 + static_cast<uint64_t>(bi) * (kBBytes >> 4);
                const uint32_t acc = (pass == 1 || i >= c.R) ? 1u : 0u;
                if (c.f8) umma_e4m3(d, ad, bd, id, acc);
                else umma_bf16(d, ad, bd, id, acc);
                r = (r + 1 == c.R) ? 0 : r + 1;
                ai = (ai + 1) & (kASlices - 1);
                bi = (bi + 1) & (kBCopies - 1);
            }
            umma_commit(bar);
            ok = mbar_wait(bar, static_cast<uint32_t>(pass), &zero, 1000000000ull);
        }
        const long long t1 = clock64();
        cycles[blockIdx.x] = ok ? static_cast<unsigned long long>(t1 - t0) : 0ull;
        if (!ok) {
            atomicExch(err, 1);
            mbar_wait(bar, 1, &zero, 1000000000ull);  // let issued UMMAs finish before TMEM is freed
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

}  // namespace

int main() {
    int sms = 0;
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0), "attribute");
    std::vector<Cfg> cases;
    // N up to 256; R ranges of 512 / R columns each must hold N
    for (int N : {16, 48, 96, 128, 192, 240, 256})
        for (int R : {1, 2, 4})
            if (R == 1 || N <= 512 / R) cases.push_back({128, N, R, 0, 4096});
    cases.push_back({64, 256, 1, 0, 4096});
    cases.push_back({64, 128, 2, 0, 4096});
    for (int N : {48, 128, 256}) cases.push_back({128, N, 1, 1, 4096});
    check(cudaFuncSetAttribute(umma_cost, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem + 1024), "attribute");
    unsigned long long *d_cycles = nullptr;
    int *d_err = nullptr;
    check(cudaMalloc(&d_cycles, sizeof(unsigned long long) * sms), "malloc");
    check(cudaMalloc(&d_err, sizeof(int)), "malloc");
    check(cudaMemset(d_err, 0, sizeof(int)), "memset");
    std::vector<unsigned long long> h(sms);
    for (const Cfg &c : cases) {
        umma_cost<<<sms, 128, kSmem + 1024>>>(c, d_cycles, d_err);
        check(cudaGetLastError(), "launch");
        check(cudaDeviceSynchronize(), "kernel");
        int herr = 0;
        check(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost), "copy");
        if (herr) {
            std::printf("TIMEOUT\n");
            return 3;
        }
        check(cudaMemcpy(h.data(), d_cycles, sizeof(unsigned long long) * sms, cudaMemcpyDeviceToHost), "copy");
        double sum = 0;
        for (unsigned long long v : h) sum += static_cast<double>(v);
        const double per = sum / sms / c.n_instr;
        const double flop = 2.0 * c.M * c.N * (c.f8 ? 32 : 16);
        std::printf("%s %d %d %d %.1f %.0f\n", c.f8 ? "e4m3" : "bf16", c.M, c.N, c.R, per, flop / per);
    }
    cudaFree(d_cycles);
    cudaFree(d_err);
    return 0;
}
