// cuBLAS DGEMM for comparison lines: native FP64, or cuBLAS's own fixed-point FP64
// emulation (CUBLAS_COMPUTE_64F_EMULATED_FIXEDPOINT, eager strategy), on row-major
// device arrays.  Built as a shared library by bench.py when nvcc is present.
//
//   int cublas_dgemm_timed(M, N, K, dA, dB, dC, emulated, mantissa_bits, reps, &ms)
//     emulated = 0: cublasGemmEx with CUBLAS_COMPUTE_64F; 1: cublasGemmEx with
//     CUBLAS_COMPUTE_64F_EMULATED_FIXEDPOINT; 2: cublasDgemm under the math mode
//     CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH (mantissa_bits > 0 fixes the retained
//     mantissa bits, 0 lets cuBLAS choose them at run time); reps timed calls after
//     one untimed call; returns 0 or a cuBLAS / CUDA status.
#include <cublas_v2.h>
#include <cuda_runtime.h>

extern "C" int cublas_dgemm_timed(int M, int N, int K, const double *dA, const double *dB, double *dC, int emulated,
                                  int mantissa_bits, int reps, float *ms) {
    cublasHandle_t h = nullptr;
    cublasStatus_t s = cublasCreate(&h);
    if (s != CUBLAS_STATUS_SUCCESS) return 1000 + static_cast<int>(s);
    void *ws = nullptr;
    const size_t ws_bytes = size_t(1) << 30;
    int rc = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const double one = 1.0, zero = 0.0;
    const cublasComputeType_t ct = emulated == 1 ? CUBLAS_COMPUTE_64F_EMULATED_FIXEDPOINT : CUBLAS_COMPUTE_64F;
    auto call = [&]() {
        // row-major C = A B is column-major C^T = B^T A^T
        if (emulated == 2) return cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &one, dB, N, dA, K, &zero, dC, N);
        return cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &one, dB, CUDA_R_64F, N, dA, CUDA_R_64F, K, &zero,
                            dC, CUDA_R_64F, N, ct, CUBLAS_GEMM_DEFAULT);
    };
    if (cudaMalloc(&ws, ws_bytes) != cudaSuccess || cublasSetWorkspace(h, ws, ws_bytes) != CUBLAS_STATUS_SUCCESS) {
        rc = 2000;
        goto done;
    }
    if (emulated) {
        if (emulated == 2 && (s = cublasSetMathMode(h, CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH)) != CUBLAS_STATUS_SUCCESS) {
            rc = 3000 + static_cast<int>(s);
            goto done;
        }
        if ((s = cublasSetEmulationStrategy(h, CUBLAS_EMULATION_STRATEGY_EAGER)) != CUBLAS_STATUS_SUCCESS) {
            rc = 3000 + static_cast<int>(s);
            goto done;
        }
        if (mantissa_bits > 0 &&
            ((s = cublasSetFixedPointEmulationMantissaControl(h, CUDA_EMULATION_MANTISSA_CONTROL_FIXED)) !=
                 CUBLAS_STATUS_SUCCESS ||
             (s = cublasSetFixedPointEmulationMaxMantissaBitCount(h, mantissa_bits)) != CUBLAS_STATUS_SUCCESS)) {
            rc = 4000 + static_cast<int>(s);
            goto done;
        }
    }
    if ((s = call()) != CUBLAS_STATUS_SUCCESS) {
        rc = 5000 + static_cast<int>(s);
        goto done;
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, nullptr);
    for (int i = 0; i < reps; ++i) call();
    cudaEventRecord(e1, nullptr);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = 6000;
        goto done;
    }
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= reps > 0 ? reps : 1;
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaDeviceSynchronize();
    if (ws) cudaFree(ws);
    cublasDestroy(h);
    return rc;
}
