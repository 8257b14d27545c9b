// Kernel variants with 32-column tiles (see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
void launch_gemm_32_3_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 3, 32>(a, g, s, st); }
void launch_gemm_32_3_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 3, 16>(a, g, s, st); }
void launch_gemm_32_4_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 4, 32>(a, g, s, st); }
void launch_gemm_32_4_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 4, 16>(a, g, s, st); }
void launch_gemm_32_5_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 5, 32>(a, g, s, st); }
void launch_gemm_32_5_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<32, 5, 16>(a, g, s, st); }
}  // namespace ozgb
