// csr.cuh - the device-resident Hamiltonian shared by assembly and the KPM kernels.
#pragma once

#include "common.cuh"

struct leo2d_csr {
  int device = 0;
  int64_t n = 0;        // orbitals (rows)
  int64_t nnz = 0;      // stored entries
  int64_t n_intra = 0;  // reference pair-list sizes (max_intra_pairs / max_inter_pairs)
  int64_t n_inter = 0;
  uint32_t flags = 0;
  leo2d::DevBuf<int64_t> rowptr;  // n + 1
  leo2d::DevBuf<int32_t> col;     // nnz
  leo2d::DevBuf<double> val64;    // nnz, FP64 values (assembly, bounds, FP64 recursion)
  leo2d::DevBuf<float> val32;     // nnz, FP32 copy streamed by the FP32 recursion
  leo2d::DevBuf<double> dx64, dy64;
  leo2d::DevBuf<float> dx32;
  leo2d::DevBuf<int32_t> grid4;   // n x 4 (i, j, orbital, sheet)
  leo2d::DevBuf<double> pos;      // n x 3
  bool has_geom = false;
  leo2d_geom geom{};
};

namespace leo2d {
// Refreshes the FP32 copies of the values from the FP64 arrays.
void csr_refresh_fp32(leo2d_ctx* ctx, leo2d_csr* csr);
}  // namespace leo2d
