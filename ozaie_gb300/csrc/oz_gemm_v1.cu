// Kernel variants with 128- and 64-column tiles (see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
void launch_gemm_128_2(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<128, 2>(a, g, s, st); }
void launch_gemm_64_3(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<64, 3>(a, g, s, st); }
void launch_gemm_64_4(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<64, 4>(a, g, s, st); }
}  // namespace ozgb
