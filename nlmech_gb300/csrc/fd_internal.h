// fd_internal.h -- device pointer bundle and launcher prototypes shared by
// the host code (fd_host.cu) and the kernel translation units.
#pragma once

#include "common.cuh"

namespace nlm {

// All node arrays are in the handle's internal (Morton) order.
struct DevPtrs {
  // geometry
  const double *pos64;  // FP64: S doubles per node (S = 2 in 2-D, 4 in 3-D)
  const float4 *pos32;  // FP32C: float4 (xh, yh, V, lo) in 2-D, (xh, yh, zh, V) in 3-D:
                        // hi = (float)x, V = nodal volume, lo = half2 of
                        // (x - hi) * lo_scale (2-D: x, y packed in .w)
  const uint2 *pos32lo; // FP32C 3-D: half2 (xl, yl), half2 (zl, 0) scaled by lo_scale
  const double *vol64;
  const float *vol32;
  const uint8_t *flags;
  const int *bcref;     // node -> BCEntry index (-1 none)
  const BCEntry *bce;
  const double *fext;   // S doubles per node, valid where FLAG_FBC is set
  // topology
  const int64_t *sell_ptr;  // per 32-node slice: first entry
  const int *sell_w;        // per slice: width (longest row)
  const int *sell_cols;     // slice-major, column-major inside a slice; -1 pads
  const int64_t *rowptr;    // CSR (n+1)
  const int *cols;          // CSR entries, rows ascending in original id
  const uint16_t *rowlen;   // row lengths
  uint32_t *bits;           // word-major bond bits: bits[w * npad + i]
  // state (ping-pong where a step reads the old and writes the new value)
  double *u64[2];  // FP64 displacement, S per node
  float4 *u32[2];  // FP32C displacement split, same shape as pos32
  double *v[2];    // FP64 velocity S per node (Verlet uses v[0]; CD ping-pongs)
  float4 *v32[2];  // FP32C velocity as a (hi, lo) FP32 pair, shape of u32
  double *f64;     // FP64 force density, S per node
  float *f32;      // FP32C force density, S per node
  // ElasticState
  const double *mw64;     // weighted volume m_i
  const float *minv32;    // FP32C: 1 / m_i formed in FP64, rounded once
  double *theta64;        // FP64: dilatation theta_i
  float2 *es_ab;          // FP32C: t = a |X| + b e coefficients per node
  int *err;               // device error flag
  const int *perm_dev;    // internal -> original node id
  // batched specimens (FP32C RNPBond): per-slice specimen id, per-specimen
  // FP32 constants (Params32) and a global table of BC time functions
  const int *slice_spec;
  const void *qtab;
  const BCTime *bct;
  // tile store (FP32C 2-D, NLM_DECOMP_TILE): per bond the index of its
  // neighbour in the tile's staged node list (the tile's kTileNodes nodes,
  // then its halo), same slice layout as sell_cols; per tile the halo ids
  const uint16_t *tile_lidx;
  // the same entries as byte offsets into a 16-byte-per-node staged array
  // (16 x index; 2-D RNPBond tile-frame kernel)
  const uint16_t *tile_boff;
  int tile_ids_bytes;    // largest id block of a tile (8 slices of tile_boff), bytes
  const int *tile_halo;  // halo lists, tile_hstride slots per tile (-1: empty)
  int tile_nmax;         // largest staged node list of any tile
  int tile_hstride;      // halo slots per tile: tile t's list is tile_halo[t * stride ...]
  // 2-D RNPBond tile-frame kernel: per node the number of leading bonds of
  // its row (a multiple of 4) whose volume factor is certainly 1, or null
  const uint8_t *row_int;
};

// Tile decomposition: kTileNodes consecutive (Morton-ordered) nodes per
// block; a tile whose node list (tile + halo) exceeds kTileMaxLocal disables
// the decomposition for the handle.
constexpr int kTileNodes = 256;
constexpr int kTileMaxLocal = 1280;
// the tile-frame kernel copies a tile's id block into shared memory; a
// store whose largest block exceeds this is not built
constexpr int kTileIdsMaxBytes = 64 * 1024;
// ElasticState tile kernels size their staged lists at run time (dynamic
// shared memory, 36 bytes per staged node); a larger tile disables them.
constexpr int kTileMaxLocalES = 3072;

// Which buffers a launch reads/writes.
struct StepArgs {
  int cur;        // index of the ping buffer holding u^m (and v^m for CD)
  bool first;     // step-0 force evaluation (no velocity completion)
  double t_now;   // t_m
  double t_next;  // t_{m+1}
  const double *tdev;  // if set: t_m = tdev[0], t_{m+1} = tdev[1] (graph replay)
  int64_t i0, i1;      // node range of this launch (FP32C RNP kernels)
  // tile decompositions: if set, the launch runs the ntiles tiles listed
  // (device array) instead of every tile
  const int *tiles;
  int64_t ntiles;
  // the launch directly follows the model's previous step on its stream (no
  // set-up kernel in between): the tile-frame kernel is then launched with
  // programmatic stream serialization, its prologue overlapping that step's
  // last blocks
  bool pdl;
};

// Launchers (return cudaError_t of the launch).
cudaError_t launch_rnp_step_fp64(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                 const StepArgs &a, int decomp, cudaStream_t s);
cudaError_t launch_rnp_step_fp32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                 const StepArgs &a, int decomp, cudaStream_t s);
cudaError_t launch_es_step_fp64(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                const StepArgs &a, int decomp, cudaStream_t s);
cudaError_t launch_es_step_fp32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                const StepArgs &a, int decomp, cudaStream_t s);
// Recompute the drift to u^{m+1} (and v^{m+1} for CD) from (u^m, v^m, f^m)
// after the host replaced the state: the second half of the step epilogue.
cudaError_t launch_drift(const StepParams &P, const DevPtrs &D, const BCTable &T, int cur,
                         double t_next, bool fp32, cudaStream_t s);
cudaError_t launch_drift32(const StepParams &P, const DevPtrs &D, const BCTable &T, int cur,
                           double t_next, cudaStream_t s);
// Banded host step (FP32C, 2-D velocity Verlet): caller-order bands in and
// out of staged copies of the caller's arrays, and the final commit.
cudaError_t launch_pipe_in32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                             double t_next, int64_t o0, int64_t o1, const int *iperm,
                             const double *hu, const double *hv, const double *hf, float4 *ua,
                             float4 *sv, float2 *sf, int *bad, cudaStream_t s);
cudaError_t launch_pipe_out32(int64_t o0, int64_t o1, const int *list, const int *iperm,
                              const float4 *ua, const float4 *sv, const float2 *sf,
                              const double *hu_in, const double *hv_in, double *ou, double *ov,
                              double *of, cudaStream_t s);
cudaError_t launch_pipe_commit32(int64_t n, int64_t nbits, const int *bad, const float4 *ua,
                                 const float4 *ub, const float4 *sv, const float2 *sf,
                                 float4 *u_now, float4 *u_next, float4 *v, float2 *f,
                                 uint32_t *bits, const uint32_t *bits_saved, cudaStream_t s);
cudaError_t launch_es_setup(const StepParams &P, const DevPtrs &D, double *mw, cudaStream_t s);
cudaError_t launch_es_minv32(const double *mw, float *minv, int64_t n, cudaStream_t s);
cudaError_t launch_damage(const StepParams &P, const DevPtrs &D, int cur, bool fp32,
                          bool es, float *phi, float *Z, cudaStream_t s);
cudaError_t launch_reaction(const StepParams &P, const DevPtrs &D, int cur, bool fp32,
                            double min_x, double max_x, double max_y, double *R, cudaStream_t s);
cudaError_t launch_energy(const StepParams &P, const DevPtrs &D, int cur, int vcur, bool fp32,
                          const double *fext, float *strain, float *work, float *kinetic,
                          float *fracture, cudaStream_t s);

}  // namespace nlm
