// Kernel variants with 128- and 64-column tiles (see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
void launch_gemm_128_2_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<128, 2, 32>(a, g, s, st); }
void launch_gemm_128_2_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<128, 2, 16>(a, g, s, st); }
void launch_gemm_64_3_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<64, 3, 32>(a, g, s, st); }
void launch_gemm_64_3_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<64, 3, 16>(a, g, s, st); }
void launch_gemm_64_4_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<64, 4, 32>(a, g, s, st); }
void launch_gemm_64_4_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<64, 4, 16>(a, g, s, st); }
}  // namespace ozgb
