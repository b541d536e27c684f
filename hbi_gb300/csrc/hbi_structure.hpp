// hbi_structure.hpp -- host-side H-matrix structure: cluster tree, leaf list
// and the device work plans derived from it.
//
// The tree and the leaf list must be bit-identical to HACApK's one-rank
// lattice H-matrix (m_HACApK_base.f90:3191-3333 tree and boxes, :2372-2460 and
// :2937-2995 admissibility, :3114-3166 leaf order).  The construction here is
// iterative (explicit stacks, node arrays) rather than recursive, but every
// arithmetic step that decides a split or an admissibility is the reference's.
#pragma once
#include <cstdint>
#include <vector>

namespace hbi {

struct Cluster {
  int nstrt = 0, nsize = 0, nnson = 0, son[2] = {-1, -1};
  double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0}, zwdth = 0;
};

// HACApK leaf record (st_HACApK_leafmtx, m_HACApK_base.f90:57-72); 1-based starts
struct Leaf {
  int ltmtx, kt, nstrtl, ndl, nstrtt, ndt;
};

struct Structure {
  int n = 0;
  std::vector<int> lod;          // lod(1:n), 1-based element ids in cluster order
  std::vector<Cluster> clusters; // node 0 is the root
  std::vector<Leaf> leaves;      // sorted by (nstrtl, nstrtt)
  std::vector<int> fine_start;   // start rows (1-based) of the finest row ranges
};

void default_params(double* p100);
// coord: coord(n,3) column-major as the reference passes it.
int build_structure(int n, const double* coord, const double* param, Structure& s);

// Row groups: the leaves that share one row range (nstrtl, ndl).  Phase 2
// gives a warp one 32-row chunk of a group and all of the group's leaves; the
// per-row sum over the (at most tree-depth) groups that cover a row follows.
struct GroupPlan {
  std::vector<int32_t> gleaf_ptr, gleaf;  // group -> its leaves, in leaf order
  std::vector<int32_t> grow0, gndl;       // 0-based first row, rows
  std::vector<int32_t> gpoff;             // offset of the group's partials
  int64_t plen = 0;                       // sum of gndl
  std::vector<int32_t> row_fc;            // row -> fine range
  std::vector<int32_t> fc_ptr, fc_group;  // fine range -> covering groups, coarse to fine
};
void plan_groups(int n, const std::vector<Leaf>& leaves, GroupPlan& gp);

// ---- streamed product plan ---------------------------------------------
// The factor store is re-laid out in row tiles of up to 32*vec rows (one
// 16-byte vector per lane, 512 bytes per column segment) so that each work
// item of the product is ONE contiguous region, which the kernels stream into
// shared memory in chunks of one stage (8 KB or 16 KB) by bulk asynchronous
// copies (TMA):
//   phase 1 (z = V^T x): the low-rank leaves sharing a column cluster form a
//     column group; item = (column group, row tile) over all its columns;
//   phase 2 (y = U z + A x): the leaves sharing a row cluster form a row group
//     (plan_groups); item = (row group, row tile) over all its columns.
// Within a region, column segments follow the group's leaf order and each
// leaf's column order; segments are padded with zeros to a multiple of vec.
// Items are ordered by decreasing size for the static warp schedule.
struct S1Item {
  int64_t soff;            // element offset of the region in the V store
  int32_t ncols, ntp;      // columns, padded rows per column
  int32_t x0, nt;          // 0-based first row of x, valid rows
  int32_t z0;              // z index of the first column
  int32_t cg;              // column group (arrival counter) when ntile > 1
  int32_t tile, ntile;     // row tile of the column group, tiles of the group
  int32_t poff;            // phase-1 partials of the group (ntile x ncols)
  int32_t cc;              // columns per streamed chunk (chunk_cols for the kernels' stage size)
};
struct S2Item {
  int64_t soff;            // element offset of the region in the U store
  int32_t ncols, ntp, nr;  // columns, padded rows, valid rows
  int32_t m0;              // multiplier index (into midx) of column 0; a multiple of 4
  int32_t pout;            // partial row sums: gpart[pout .. pout+nr)
  int32_t cc;              // columns per streamed chunk
};
struct SegCopy {           // conversion of one column segment from the FP64 body
  int64_t dst, src;        // element offsets (dst in the V or U store)
  int32_t len, stride;     // valid rows, source element stride between rows
  int32_t swz, pad;        // XOR mask of the 16-byte vector index (vswz), 0 = none
};
struct StreamPlan {
  int vec = 1, tr = 1;
  std::vector<S1Item> p1;
  std::vector<S2Item> p2;
  int64_t vstore = 0, ustore = 0;    // elements
  int64_t zlen = 0, plen1 = 0, ncg = 0, plen2 = 0;
  std::vector<int32_t> midx;         // per row-group column: z index, or -(x index)-1; groups padded to 4
  GroupPlan gp;                      // row groups, fine ranges
  std::vector<int32_t> gnch;         // partial columns per row group (1)
  std::vector<int32_t> gpoff2;       // partial offset per row group
  // phase 3: fine range f -> fcb_base[fcb_ptr[f] .. fcb_ptr[f+1]), the
  // partial of row r in each non-empty covering group at fcb_base + r,
  // coarse to fine
  std::vector<int32_t> fcb_ptr, fcb_base;
  std::vector<SegCopy> vcopy, ucopy; // conversion maps
  int64_t factor_elems = 0;
};
// XOR mask of the 16-byte vectors of column c in a V-store segment of nv
// vectors: within each aligned group of g = gcd(nv, 8) vectors, vector k of
// column c is stored at k ^ vswz(c, nv).  Eight consecutive columns read at
// the same logical vector then fall on eight different 16-byte bank slots of
// shared memory (c * nv + (k ^ s) is distinct mod 8 over c), so a warp whose
// lanes own consecutive columns reads a stage without bank conflicts.  The
// mask only depends on c mod 8, and chunks start at multiples of 16 columns.
#if defined(__CUDACC__)
__host__ __device__
#endif
inline int vswz(int c, int nv) {
  const int g = (nv & -nv) < 8 ? (nv & -nv) : 8;
  const int shift = g == 8 ? 0 : g == 4 ? 1 : g == 2 ? 2 : 3;
  return (c >> shift) & (g - 1);
}

// columns of one streamed chunk in a shared-memory stage of stage_bytes (8 KB
// or 16 KB): as many whole columns as fit, a multiple of 16 (ntp * esz <= 512,
// so at least 16), and at most 128 (four phase-2 multipliers per lane)
#if defined(__CUDACC__)
__host__ __device__
#endif
inline int chunk_cols(int ntp, int esz, int stage_bytes) {
  const int c = (stage_bytes / (ntp * esz)) / 16 * 16;
  return c < 128 ? c : 128;
}
// Static schedule of one phase's items over nwarps warps: longest
// processing time first -- items in decreasing cost, each to the warp with
// the least work so far (ties to the lower warp); a warp keeps its items in
// that order.  woff (nwarps + 1) and witem are its CSR lists.
void plan_warp_schedule(const std::vector<int64_t>& cost, int nwarps, std::vector<int32_t>& woff,
                        std::vector<int32_t>& witem);
// Static schedule with locality: the items in order of `key` (their offset
// in the store) are cut into nblocks consecutive runs of near-equal cost, and
// each run is dealt over its block's nw warps longest first.  A block then
// streams one compact region of the store instead of items from all over it.
// woff (nblocks * nw + 1) and witem as plan_warp_schedule, warp b * nw + w.
void plan_block_schedule(const std::vector<int64_t>& cost, const std::vector<int64_t>& key, int nblocks, int nw,
                         std::vector<int32_t>& woff, std::vector<int32_t>& witem);

// ---- tensor-core plan of the ensemble product ---------------------------
// Both contractions as D (64 members x N) = A (64 x K) * B^T with B (N x K)
// from the factor store: phase 2 N = the rows of a row-group tile (<= 256),
// K = the group's columns; phase 1 N = the columns of a column group (<= 256
// per item), K = the rows of a tile (<= kTcK1).  B is stored as BF16 hi + lo
// halves (x = hi + lo to ~16 bits) in the canonical no-swizzle K-major layout,
// per 16-K chunk: [hi: 2 K-blocks x N/8 core matrices of 8 x 8][lo: same].
// N is padded to 8 and K to 16 with zeros.
constexpr int kTcK1 = 1024;  // rows of a phase-1 tile (K of one item)
struct TcItem {
  int64_t soff;            // bf16 element offset of the item's first chunk
  int32_t np, kp;          // N padded to 8, K padded to 16
  int32_t nv, kv;          // valid N, valid K
  int32_t m0;              // phase 2: midx of column 0; phase 1: x row of K index 0
  int32_t out0;            // phase 2: gpart row offset; phase 1: z index of column 0
  int32_t cg, tile, ntile, poff;  // phase 1 multi-tile reduction (as S1Item)
  int32_t pad[2];
};
struct TcCopy {            // one run of a column (or tile-row) from the FP64 body
  int64_t item, src;       // bf16 offset of the item, body offset of element 0
  int32_t np;              // the item's padded N
  int32_t n0, k0;          // canonical (n, k) of element 0
  int32_t dn, dk;          // step per element along n and k (one of them 0)
  int32_t len, stride;     // elements, body stride
};
struct TcPlan {
  std::vector<TcItem> p1, p2;
  int64_t store1 = 0, store2 = 0;  // bf16 elements (hi and lo halves included)
  int64_t zlen = 0, plen1 = 0, ncg = 0;
  std::vector<int32_t> midx;       // as StreamPlan::midx
  std::vector<TcCopy> copy1, copy2;
};
void plan_tc(int n, const std::vector<Leaf>& leaves, const std::vector<int64_t>& body_off, TcPlan& tp);

// body_off: element offset of each leaf in the HACApK FP64 body (low rank:
// [V ndt x kt][U ndl x kt] column-major; dense a1(ndt, ndl))
// stage_bytes: the phase kernels' shared-memory stage (8 KB or 16 KB), which
// sets each item's chunk width cc
void plan_stream(int n, const std::vector<Leaf>& leaves, const std::vector<int64_t>& body_off, int vec,
                 StreamPlan& sp, int stage_bytes = 8192);

}  // namespace hbi
