// csr.cuh - the device-resident Hamiltonian shared by assembly and the KPM kernels.
#pragma once

#include "common.cuh"

namespace leo2d {
// Elements allocated past the end of rowptr / col / val so that bulk copies of
// a tile may round their range up to 16-byte multiples without leaving the
// allocation. The padding is zero-filled.
constexpr int64_t kCsrPad = 16;
}  // namespace leo2d

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
  leo2d::DevBuf<float> val32;     // nnz, FP32 copy of the values
  leo2d::DevBuf<uint2> ent;       // nnz, (column, FP32 value bits) streamed by the FP32 recursion
  leo2d::DevBuf<uint2> entd;      // nnz, (column, FP32 dxH bits)
  leo2d::DevBuf<double> dx64, dy64;
  bool complex_h = false;         // Peierls phases: entries have imaginary parts
  // a field on a periodic supercell: the reference's Peierls phase on the
  // images (x1 shifted by the image, locality.cpp:4718-4738, 7157-7161) breaks
  // Hermiticity, so the moments below P/2 are taken directly (see run_trace)
  bool nonhermitian = false;
  leo2d::DevBuf<double> val_im64; // nnz, FP64 imaginary parts (complex_h)
  leo2d::DevBuf<float> val_im32;  // nnz, FP32 copy
  leo2d::DevBuf<float> dx32;
  leo2d::DevBuf<int32_t> grid4;   // n x 4 (i, j, orbital, sheet)
  leo2d::DevBuf<double> pos;      // n x 3
  bool has_geom = false;
  leo2d_geom geom{};
  // largest stored-entry count of any tile of `tile_rows` consecutive rows (cached)
  int tile_rows_cached = 0;
  int64_t tile_max_nnz = 0;
  // locality-ordered copy streamed by the recursion (reorder.cu)
  bool reordered = false;
  bool reorder_fp64 = false;
  double reorder_patch = 0.0;
  int reorder_curve = 0;          // 1: patch, sheet, then a fine Hilbert curve inside the patch
  int reorder_curve_req = -1;     // the curve setting the copy was built for (may fall back to 0)
  leo2d::DevBuf<int32_t> new2old, old2new;
  leo2d::DevBuf<int64_t> prow;
  leo2d::DevBuf<int32_t> pcol;
  leo2d::DevBuf<float> pval32;
  leo2d::DevBuf<uint2> pent;
  leo2d::DevBuf<double> pval64;
  leo2d::DevBuf<float> pval_im32;   // permuted FP32 imaginary parts (complex_h)
  int perm_tile_rows = 0;
  int64_t perm_tile_max_nnz = 0;
  // tensor-core tiles of the locality-ordered copy (tc_spmm.cu): for each tile
  // of 128 rows the sorted distinct columns (its window, <= 1024), and each
  // row's entries as (window position, FP32 value) sorted by position
  bool tc_built = false;
  double tc_patch = 0.0;
  int64_t tc_tiles = 0;
  int tc_max_ent = 0;                 // most entries in one tile
  int tc_max_win = 0;                 // widest window
  double tc_mean_win = 0.0;
  leo2d::DevBuf<int32_t> tc_win;      // [tiles][1024] window rows, padded with the last row
  leo2d::DevBuf<int32_t> tc_nwin;     // [tiles] window width
  leo2d::DevBuf<uint2> tc_ent;        // nnz (+pad): (position, value bits), rows as prow
  leo2d::DevBuf<uint8_t> tc_cstart;   // [n][16] first entry of each 64-position chunk, from the row start
  // row blocks of the locality-ordered copy (rb_spmm.cu): blocks of 4 rows, each
  // the sorted union of its rows' columns (slots) with a dense 4 x slots panel
  bool rb_built = false;
  double rb_patch = 0.0;
  int64_t rb_blocks = 0;              // row blocks
  int64_t rb_slots = 0;               // slots stored (padded to multiples of 4 per block)
  int64_t rb_union = 0;               // slots before padding
  int rb_max_slots = 0;               // most slots of one block (before padding)
  int rb_tile_warps = 0;              // tile width (blocks) of rb_tile_max_bytes (the last one asked for)
  int64_t rb_tile_max_bytes = 0;      // largest tile of rb_tile_warps blocks (data bytes)
  int64_t rb_tile_bytes_w[5] = {};    // the same per tile width 8 w (w = 1..4), 0: not measured
  leo2d::DevBuf<int64_t> rb_off;      // [blocks + 1 + pad] first slot of each block
  leo2d::DevBuf<unsigned char> rb_data;  // 20 bytes per slot: columns, then the value panel
  leo2d::DevBuf<float> rb_im;         // [slots][4] imaginary value panel (complex_h)
  bool rb_xs_built = false;           // positions for the velocity step (Kubo)
  leo2d::DevBuf<float> rb_xrel;       // [blocks][4] x of each row minus x of its block's first row
  leo2d::DevBuf<float> rb_xs;         // [slots] x of the slot's column minus the same
  // row blocks of 8 or 16 rows for the tensor-core step (rt_spmm.cu): the union
  // of each block's columns in k-steps of 8 slots, stored in the processing
  // order of one launch shape (warps, group, chunk, grid)
  int rt_rows = 0;                    // rows per block of the counted / built blocks
  bool rt_counted = false;            // rt_kst holds the k-steps of every block
  bool rt_built = false;
  double rt_patch = 0.0;              // ordering the blocks were built from
  int rt_curve = -1;
  int64_t rt_blocks = 0;
  int64_t rt_ksteps = 0;              // k-steps stored
  int64_t rt_union = 0;               // slots before padding
  int rt_max_slots = 0;
  int rt_warps = 0, rt_group = 0, rt_chunk = 0;
  unsigned rt_grid = 0;
  leo2d::DevBuf<int64_t> rt_kst;      // [blocks] k-steps of each block
  leo2d::DevBuf<int64_t> rt_wbeg;     // [grid * warps + 1] first k-step of each warp
  leo2d::DevBuf<unsigned char> rt_data;  // 32 + 32 rt_rows bytes per k-step
  // shared-memory windows of the row blocks (rbw_spmm.cu): per tile of 16 blocks
  // the sorted distinct columns of its slots; slots hold window positions
  bool rbw_built = false;
  int64_t rbw_tiles = 0;
  int rbw_max_win = 0;                // widest window (rows)
  int64_t rbw_win_rows = 0;           // window rows over all tiles
  int64_t rbw_tile_max_bytes = 0;     // largest tile's slots (bytes)
  int64_t rbw_runs_total = 0;         // runs over all tiles
  leo2d::DevBuf<int64_t> rbw_roff;    // [tiles + 1] first run of each tile
  leo2d::DevBuf<int32_t> rbw_runs;    // (first column, rows) per run
  leo2d::DevBuf<int32_t> rbw_wrows;   // [tiles] window rows
  leo2d::DevBuf<unsigned char> rbw_data;  // rb_data with window positions over the columns
};

namespace leo2d {
// Refreshes the FP32 copies of the values from the FP64 arrays.
void csr_refresh_fp32(leo2d_ctx* ctx, leo2d_csr* csr);
// Allocates rowptr (n+1), col and val64 (nnz) with zeroed kCsrPad padding.
void csr_alloc_rowptr(leo2d_ctx* ctx, leo2d_csr* csr, int64_t n);
void csr_alloc_entries(leo2d_ctx* ctx, leo2d_csr* csr, int64_t nnz, bool with_dx);
// Builds / drops the locality-ordered copy (patch = real-space patch edge, A;
// curve: inside a patch by sheet, then along a Hilbert curve of 1/32-patch
// cells, else by the reference index).
void csr_build_reordered(leo2d_ctx* ctx, leo2d_csr* csr, double patch, bool with_fp64, bool curve = false);
// Per-orbital disregistry (Hstruct::getShiftConfigs) into device memory out[n][2]; bilayers.
void csr_shift_configs(leo2d_ctx* ctx, const leo2d_csr* csr, double* out);
void csr_drop_reordered(leo2d_csr* csr);
// Builds the tensor-core tiles of the locality-ordered copy; returns false (and
// builds nothing) when a tile has more than 1024 distinct columns, 16384
// entries or a row of more than 255 entries.
bool csr_build_tc(leo2d_ctx* ctx, leo2d_csr* csr);
void csr_drop_tc(leo2d_csr* csr);
// Builds the row blocks of the locality-ordered copy; returns false (and builds
// nothing) when a block of 4 rows has more than 4096 entries or 2048 distinct columns.
bool csr_build_rb(leo2d_ctx* ctx, leo2d_csr* csr);
void csr_drop_rb(leo2d_csr* csr);
// x positions of the ordered rows and of every row-block slot's column relative
// to the block's first row (the velocity step's D_ij = (x_i - x_j) H~_ij); once
// per matrix.
void csr_build_rb_xs(leo2d_ctx* ctx, leo2d_csr* csr);
// Largest data bytes of a tile of `tile` consecutive row blocks.
int64_t rb_tile_max_bytes(leo2d_ctx* ctx, const leo2d_csr* csr, int tile);
// Builds the row blocks (8 or 16 rows) of the tensor-core step for one launch
// shape (max_grid > 0: at most that many CTAs walk them, else one per SM);
// returns false (and builds nothing) when a block holds more than 2048 stored
// entries.
bool csr_build_rt(leo2d_ctx* ctx, leo2d_csr* csr, int warps, int group, int chunk, int rows, int max_grid = 0);
void csr_drop_rt(leo2d_csr* csr);
// Builds the shared-memory windows of the row blocks; returns false (and builds
// nothing) when a tile of 16 blocks has more than 8192 slots or 2048 distinct columns.
bool csr_build_rbw(leo2d_ctx* ctx, leo2d_csr* csr);
void csr_drop_rbw(leo2d_csr* csr);
}  // namespace leo2d
