// Kernel variants with 48-column tiles (see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
void launch_gemm_48_3_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<48, 3, 32>(a, g, s, st); }
void launch_gemm_48_3_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<48, 3, 16>(a, g, s, st); }
void launch_gemm_48_4_32(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<48, 4, 32>(a, g, s, st); }
void launch_gemm_48_4_16(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<48, 4, 16>(a, g, s, st); }
}  // namespace ozgb
