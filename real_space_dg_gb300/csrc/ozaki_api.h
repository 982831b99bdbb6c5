// FP64 GEMM emulated on the BF16 tensor cores (ozaki.cuh) as a building block for
// other operators: C (M x Ncol, column-major, ldc = M) += A (M x K, row-major, fixed,
// digit-sliced once on the host) * X (K x Ncol, column-major: K consecutive doubles per
// column, sliced on the device at every call).  K <= 1024; the digit rows are padded to
// a multiple of 8 for the 16-byte TMA rows.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace wg {

struct OzakiRowsDev {
  __nv_bfloat16* dig = nullptr;   // [8][M][Kp]
  int* e = nullptr;               // [M] row exponents
  CUtensorMap map;
  int M = 0, K = 0, Kp = 0;
};

struct OzakiColsDev {
  __nv_bfloat16* dig = nullptr;   // [8][Ncol][Kp]
  int* e = nullptr;               // [Ncol]
  CUtensorMap map;
  long long ncol = 0;
  int Kp = 0;
};

int ozaki_rows_upload(const std::vector<double>& A, int M, int K, OzakiRowsDev& out, std::string& err);
int ozaki_cols_alloc(long long ncol, int K, OzakiColsDev& out, std::string& err);
void ozaki_free(OzakiRowsDev& a);
void ozaki_free(OzakiColsDev& b);
// C += A X; err: device flag raised when a bounded barrier wait of the GEMM times out.
cudaError_t ozaki_accumulate(const OzakiRowsDev& A, OzakiColsDev& B, const double* X, double* C, int* err,
                             cudaStream_t st);
// C = A X (overwrites C).
cudaError_t ozaki_multiply(const OzakiRowsDev& A, OzakiColsDev& B, const double* X, double* C, int* err,
                           cudaStream_t st);

}  // namespace wg
