// fec_pattern.h -- the symbolic phase on the device: node adjacency, sorted
// neighbour lists, CSC column lengths and offsets, the element map, and the CSC
// pattern itself (the reference's SparseMatrixPattern + _update_dofs! and the
// colptr/rowval of sparse!, src/assemblers/SparsityPatterns.jl:53-231,301-308).
//
// Every output equals what the host symbolic phase (fec_pattern_build) forms:
// adjacency entries in increasing element order, neighbour lists sorted and
// unique, rows of a column in increasing unknown order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fec {

constexpr int PATTERN_MAX_BLOCKS = 16;  // element blocks the device build handles
constexpr int PATTERN_CAND_CAP = 2048;  // adjacent-element nodes gathered per node (before de-duplication)

struct PatternBlocks {
  int nblocks;
  int nnpe[PATTERN_MAX_BLOCKS];
  int64_t ne[PATTERN_MAX_BLOCKS], elem_start[PATTERN_MAX_BLOCKS], conn_off[PATTERN_MAX_BLOCKS],
      epos_off[PATTERN_MAX_BLOCKS];
};

// cnt[n] += number of (element, local node) entries of node n, all blocks.
cudaError_t pattern_count_adjacency(const int32_t* conn, int64_t n_entries, int32_t* cnt, cudaStream_t s);
// out[0] = 0, out[i + 1] = in[0] + ... + in[i] (int64); scratch >= pattern_scan_scratch(n) int64.
size_t pattern_scan_scratch(int64_t n);
cudaError_t pattern_scan(const int32_t* in32, const int64_t* in64, int64_t n, int64_t* out, int64_t* scratch,
                         cudaStream_t s);
// nadj[ptr[n] ...] = (global element << 5) | local node, then each node's run sorted.
cudaError_t pattern_fill_adjacency(const PatternBlocks& B, const int32_t* conn, const int64_t* ptr, int64_t nn,
                                   int32_t* cursor, uint32_t* nadj, cudaStream_t s);
// Pass 1 (nbr == nullptr): nbr_cnt[n], col_len[n] (unknown rows per column).
// Pass 2: the sorted unique neighbour list and each neighbour's row offset.
// *err gets 1 if a node gathers more than PATTERN_CAND_CAP nodes.
cudaError_t pattern_neighbours(const PatternBlocks& B, const int32_t* conn, const int64_t* adj_ptr,
                               const uint32_t* nadj, int64_t nn, const uint8_t* umask, int32_t* nbr_cnt,
                               int32_t* col_len, const int64_t* nbr_ptr, int32_t* nbr, int32_t* rowoff, int* err,
                               cudaStream_t s);
// w[n] = (unknown components of n) * col_len[n]; *max_len = max col_len, *max_cols = max w.
cudaError_t pattern_column_sizes(int64_t nn, const uint8_t* umask, const int32_t* col_len, int64_t* w,
                                 int* max_len, int* max_cols, cudaStream_t s);
// epos[e][a][b] = row offset of node conn[b] inside node conn[a]'s columns.
cudaError_t pattern_element_map(const PatternBlocks& B, const int32_t* conn, const int64_t* nbr_ptr,
                                const int32_t* nbr, const int32_t* rowoff, uint16_t* epos, cudaStream_t s);
// umask_out[n] = umask[n] | full_flag when n and every neighbour have all nf components unknown.
cudaError_t pattern_full_neighbourhood(int64_t nn, int nf, const int64_t* nbr_ptr, const int32_t* nbr,
                                       const uint8_t* umask, uint8_t full_flag, uint8_t* umask_out, cudaStream_t s);
// 1-based CSC colptr (n_unknowns + 1) and rowval (nnz) over the unknowns.
cudaError_t pattern_csc(int64_t nn, int nf, const uint8_t* umask, const int64_t* dof_to_unknown,
                        const int64_t* nbr_ptr, const int32_t* nbr, const int64_t* col_base, const int32_t* col_len,
                        int64_t* colptr, int64_t* rowval, cudaStream_t s);

}  // namespace fec
