// Cost of back-to-back tcgen05.mma instructions (cta_group::1, M = 128, K = 16,
// bf16) on this GPU, as the slice-pair GEMM's planner models it.  One CTA per SM;
// operands change from one instruction to the next; SM cycles per instruction are
// measured with clock64 from the first issue to the commit's arrival.
//
//   tight: one thread issues n UMMAs of width N from a minimal loop (the rate of
//          the tensor pipe for wide N, the issuing thread's rate for narrow N);
//   pairs: the 43 UMMAs of one K step of 8 slices with the pair set p + q <= 8,
//          one per slice pair into its bin's accumulator range, N = 48, dealt
//          to one or two issuing warps (on different schedulers).
//
// Prints one line per case:  mode N issuers cycles_per_umma
// Every wait on a commit's mbarrier is bounded (1 s); a timeout prints TIMEOUT and
// the program exits 3 after the kernel has released TMEM.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../ozaie_gb300/csrc/oz_ptx.cuh"

using namespace ozgb;

namespace {

constexpr int kSmem = 160 * 1024;
constexpr int kTight = 0, kPairs = 1;

struct Cfg {
    int mode, N, issuers, n_instr;
};

__global__ void __launch_bounds__(128, 1) umma_cost(const Cfg c, unsigned long long *out, int *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *Ab = smem;              // 8 A slices of 128 rows x 32 B
    uint8_t *Bb = smem + 32 * 1024;  // up to 64 KB of B rows x 32 B
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 96 * 1024);  // [2]
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 2);
    for (int i = threadIdx.x * 16; i < 96 * 1024; i += blockDim.x * 16)
        *reinterpret_cast<uint4 *>(smem + i) = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
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
    // issuing threads: lane 0 of warps 1 and 2 (schedulers 1 and 2)
    const int iss = threadIdx.x == 32 ? 0 : (threadIdx.x == 64 ? 1 : -1);
    if (iss >= 0 && iss < c.issuers) {
        const uint32_t id = idesc_bf16_f32(128, c.N);
        const uint64_t a0 = smem_desc(smem_u32(Ab), 128, 256);
        const uint64_t b0 = smem_desc(smem_u32(Bb), 128, 256);
        const int zero = 0;
        bool ok = true;
        long long t0 = 0, issued = 0;
        for (int pass = 0; pass < 2 && ok; ++pass) {  // pass 0 warms up
            if (pass == 1) {
                t0 = clock64();
                issued = 0;
            }
            if (c.mode == kTight) {
                int ai = 0, bi = 0;
                for (int i = 0; i < c.n_instr; ++i) {
                    umma_bf16(tmem, a0 + static_cast<uint64_t>(ai) * 256, b0 + static_cast<uint64_t>(bi) * 512, id,
                              (pass == 1 || i > 0) ? 1u : 0u);
                    ai = (ai + 1) & 7;
                    bi = (bi + 1) & 3;
                }
                issued = c.n_instr;
            } else {
                // bin p + q at TMEM columns (p + q) N; B slice q at q N rows
                const uint32_t b_step = (c.N * 32) >> 4;
                const int ksteps = c.n_instr / 43;
                for (int k = 0; k < ksteps; ++k) {
                    for (int p = iss; p < 8; p += c.issuers) {
                        const uint64_t ad = a0 + static_cast<uint64_t>(p) * 256;
                        const int qmax = 8 - p < 7 ? 8 - p : 7;
                        uint32_t d = tmem + static_cast<uint32_t>(p * c.N);
                        uint64_t bd = b0;
                        for (int q = 0; q <= qmax; ++q) {
                            umma_bf16(d, ad, bd, id, (pass == 1 || k > 0) ? 1u : 0u);
                            d += c.N;
                            bd += b_step;
                        }
                        issued += qmax + 1;
                    }
                }
            }
            umma_commit(&bar[iss]);
            ok = mbar_wait(&bar[iss], static_cast<uint32_t>(pass), &zero, 1000000000ull);
        }
        const long long t1 = clock64();
        out[4 * blockIdx.x + 2 * iss] = ok ? static_cast<unsigned long long>(t1 - t0) : 0ull;
        out[4 * blockIdx.x + 2 * iss + 1] = static_cast<unsigned long long>(issued);
        if (!ok) {
            atomicExch(err, 1);
            mbar_wait(&bar[iss], 1, &zero, 1000000000ull);  // let issued UMMAs finish before TMEM is freed
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
    // shared memory: A 32 KB; B 4 copies of up to 8 KB (tight) or 8 slices of N x 32 B (pairs)
    for (int N : {16, 48, 96, 128, 192, 256}) cases.push_back({kTight, N, 1, 8192});
    for (int ni : {1, 2}) cases.push_back({kPairs, 48, ni, 43 * 256});
    check(cudaFuncSetAttribute(umma_cost, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem), "attribute");
    unsigned long long *d_out = nullptr;
    int *d_err = nullptr;
    check(cudaMalloc(&d_out, sizeof(unsigned long long) * 4 * sms), "malloc");
    check(cudaMalloc(&d_err, sizeof(int)), "malloc");
    check(cudaMemset(d_err, 0, sizeof(int)), "memset");
    std::vector<unsigned long long> h(4 * sms);
    for (const Cfg &c : cases) {
        check(cudaMemset(d_out, 0, sizeof(unsigned long long) * 4 * sms), "memset");
        umma_cost<<<sms, 128, kSmem>>>(c, d_out, d_err);
        check(cudaGetLastError(), "launch");
        check(cudaDeviceSynchronize(), "kernel");
        int herr = 0;
        check(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost), "copy");
        if (herr) {
            std::printf("TIMEOUT\n");
            return 3;
        }
        check(cudaMemcpy(h.data(), d_out, sizeof(unsigned long long) * 4 * sms, cudaMemcpyDeviceToHost), "copy");
        double cyc = 0, n = 0;
        for (int i = 0; i < sms; ++i) {
            double m = 0;
            for (int j = 0; j < c.issuers; ++j) {
                m = static_cast<double>(h[4 * i + 2 * j]) > m ? static_cast<double>(h[4 * i + 2 * j]) : m;
                n += static_cast<double>(h[4 * i + 2 * j + 1]);
            }
            cyc += m;
        }
        std::printf("%s %d %d %.1f\n", c.mode == kTight ? "tight" : "pairs", c.N, c.issuers, cyc / n);
    }
    cudaFree(d_out);
    cudaFree(d_err);
    return 0;
}
