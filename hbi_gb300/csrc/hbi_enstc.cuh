// hbi_enstc.cuh -- the ensemble's tensor-core product: device view of one
// H-matrix's tensor-core stores and the launchers (hbi_enstc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "hbi_structure.hpp"

namespace hbi {

struct TcMat {            // one H-matrix's tensor-core stores and ensemble scratch
  const TcItem* p1;
  int n1;
  const TcItem* p2;
  int n2;
  const __nv_bfloat16* s1;  // phase-1 store
  const __nv_bfloat16* s2;  // phase-2 store
  const int32_t* midx;
  float* z;                 // zlen x 64
  float* part;              // plen1 x 64
  int* cnt;                 // per column group piece
  float* gpart;             // rows of the row groups x 64 (the operator's phase-3 layout)
  int* err;
  long long wait;           // bound of a wait (SM clock cycles; 0: every wait gives up), the operator's
  // static schedule of both matrices' items over G blocks (first matrix's
  // view only): block b walks bitem[ph][boff[ph][b] .. boff[ph][b + 1]),
  // item i < n of the first matrix, else item i - n of the second
  const int32_t* boff[2];
  const int32_t* bitem[2];
  int G;
};

size_t tc_smem_bytes();
void tc_prepare();
void launch_tc(int phase, const TcMat& a, const TcMat& b, int nmat, const float* x, cudaStream_t st);
void launch_tcconv(const double* body, const TcCopy* map, int64_t nmap, __nv_bfloat16* dst, cudaStream_t st);

}  // namespace hbi
