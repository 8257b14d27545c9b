// Kernel variants with 32- and 16-column tiles (see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
void launch_gemm_32_4(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 4>(a, g, s, st); }
void launch_gemm_32_5(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 5>(a, g, s, st); }
void launch_gemm_16_4(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<16, 4>(a, g, s, st); }
void launch_gemm_16_5(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<16, 5>(a, g, s, st); }
}  // namespace ozgb
