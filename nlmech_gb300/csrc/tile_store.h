// tile_store.h -- building the tile store of the tile decompositions (one
// model or a batch's combined layout).
#pragma once

#include "fd_handle.h"

namespace nlm {

// Tile store of NLM_DECOMP_TILE (FP32C, 2-D): tile t = internal nodes
// [256 t, 256 t + 256); its halo = the nodes outside the tile its rows
// reach, ascending.  Each bond stores its neighbour's index in the tile's
// staged list (tile nodes 0..255, halo from 256), in the sliced layout of
// sell_cols; padding entries point at the row's own node.  If some tile needs
// more than kTileMaxLocal staged nodes the store is not built.  The 2-D
// RNPBond store (max_local == kTileMaxLocal) also gets the byte-offset copy
// tile_boff (16 x index).  With lattice residues (lres: a lattice-renumbered
// model) the halo is laid out by residue: halo node j takes staged slot
// 256 + 8 m + res(j) (m counting the tile's halo nodes of that residue), so
// that eight neighbours of one lattice offset from a quarter warp's 4 x 2
// patch (2 x 2 x 2 block in 3-D) land in eight different 16-byte bank
// groups; the slots left empty hold -1 in the halo list and are skipped by
// the staging.
// What a tile store is built from (one model or a batch's combined layout).
struct TileInputs {
  int64_t n, nnz, nslices, sell_entries;
  const int *cols_dev;                 // internal column ids, CSR order
  const int64_t *sell_ptr_dev;         // sliced-store offsets
  const std::vector<int64_t> *rowptr;  // host CSR offsets
  const std::vector<int> *perm;        // internal -> caller id (for tile_need), or null
  int max_local;                       // largest staged list allowed
  const std::vector<uint8_t> *lres = nullptr;  // lattice residues per node, or null
  // interior prefixes (2-D RNPBond store): caller-order positions (3 per
  // node, with perm), the radius below which a bond is certainly outside
  // the volume-correction band, and the largest tile extent for which the
  // tile frame's rounding stays far below the margin in that radius
  const double *xc = nullptr;
  double r_int = 0., ext_max = 0.;
  // or: positions in the internal order (xs doubles per node) and a radius
  // per node (a batch of specimens with their own mesh sizes)
  const double *xin = nullptr;
  int xs = 3;
  const double *r_int_node = nullptr;
};

template <class H>
int build_tile_store(H *h, const TileInputs &in, bool &ok, std::vector<int> *need_out) {
  const int64_t n = in.n, nt = (n + kTileNodes - 1) / kTileNodes;
  const int max_local = in.max_local;
  ok = false;
  std::vector<int> cols(in.nnz);
  std::vector<int64_t> sptr(in.nslices + 1);
  NLM_CUDA(cudaMemcpyAsync(cols.data(), in.cols_dev, sizeof(int) * in.nnz, cudaMemcpyDeviceToHost,
                           h->stream));
  NLM_CUDA(cudaMemcpyAsync(sptr.data(), in.sell_ptr_dev, sizeof(int64_t) * (in.nslices + 1),
                           cudaMemcpyDeviceToHost, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  const std::vector<int64_t> &rp = *in.rowptr;
  std::vector<std::vector<int>> halo(nt);
  const bool boff_too = max_local == kTileMaxLocal;
  std::vector<uint16_t> lidx(in.sell_entries + 4, 0);
  std::vector<uint16_t> boff(boff_too ? in.sell_entries + 4 : 0, 0);
  std::vector<int> too_big(1, 0);
  // per node: how many leading bonds of its row (whole groups of four) lie
  // within r_int, where the volume factor min(1, (check_up - r) / h) is 1
  const bool rint_too =
      boff_too && ((in.xc && in.perm && in.r_int > 0.) || (in.xin && in.r_int_node));
  std::vector<uint8_t> rint(rint_too ? n : 0, 0);
  std::vector<int> need(nt, -1);
  std::vector<std::vector<int>> halo_slots(nt);  // lattice layout: halo by slot, -1 = empty
  unsigned nthr = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  auto work = [&](unsigned w) {
    for (int64_t t = w; t < nt; t += nthr) {
      const int64_t a = t * kTileNodes, b = std::min(n, a + kTileNodes);
      std::vector<int> &hl = halo[t];
      for (int64_t q = rp[a]; q < rp[b]; q++)
        if (cols[q] < a || cols[q] >= b) hl.push_back(cols[q]);
      std::sort(hl.begin(), hl.end());
      hl.erase(std::unique(hl.begin(), hl.end()), hl.end());
      if (in.perm) {
        int m = -1;
        for (int64_t i = a; i < b; i++) m = std::max(m, (*in.perm)[i]);
        for (int j : hl) m = std::max(m, (*in.perm)[j]);
        need[t] = m;
      }
      // staged slot (from kTileNodes) of each halo node, in hl's order
      std::vector<int> hslot(hl.size());
      for (size_t k = 0; k < hl.size(); k++) hslot[k] = (int)k;
      if (in.lres) {
        int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (size_t k = 0; k < hl.size(); k++) {
          const int r = (*in.lres)[hl[k]] & 7;
          hslot[k] = 8 * cnt[r]++ + r;
        }
        int m = 0;
        for (int r = 0; r < 8; r++) m = std::max(m, cnt[r]);
        std::vector<int> bys(8 * (size_t)m, -1);
        for (size_t k = 0; k < hl.size(); k++) bys[hslot[k]] = hl[k];
        // the sorted list is needed below for lookups: keep it, store the
        // slot-ordered one after the rows are written
        halo_slots[t] = std::move(bys);
      }
      const int64_t nstaged = in.lres ? (int64_t)halo_slots[t].size() : (int64_t)hl.size();
      if (kTileNodes + nstaged > max_local) {
        too_big[0] = 1;
        continue;
      }
      if (rint_too) {
        auto X = [&](int64_t k) {
          return in.xin ? in.xin + (int64_t)in.xs * k : in.xc + 3 * (int64_t)(*in.perm)[k];
        };
        const double *xo = X(a);
        double ext = 0.;
        for (int64_t i = a; i < b; i++) {
          const double *xi = X(i);
          ext = std::max(ext, std::max(std::fabs(xi[0] - xo[0]), std::fabs(xi[1] - xo[1])));
          for (int64_t q = rp[i]; q < rp[i + 1]; q++) {
            const double *xj = X(cols[q]);
            ext = std::max(ext, std::max(std::fabs(xj[0] - xo[0]), std::fabs(xj[1] - xo[1])));
          }
        }
        // the split (hi, lo) positions carry ~2^-35 of |x|: keep that far
        // below the margin too
        const bool near = std::max(std::fabs(xo[0]), std::fabs(xo[1])) <= 1000. * in.ext_max;
        if (ext <= in.ext_max && near)
          for (int64_t i = a; i < b; i++) {
            const double *xi = X(i);
            const double ri = in.r_int_node ? in.r_int_node[i] : in.r_int;
            int64_t k = 0;
            for (int64_t q = rp[i]; q < rp[i + 1] && k < 252; q++, k++) {
              const double *xj = X(cols[q]);
              if (!(std::hypot(xj[0] - xi[0], xj[1] - xi[1]) <= ri)) break;
            }
            rint[i] = (uint8_t)(k & ~int64_t(3));
          }
      }
      for (int64_t i = a; i < b; i++) {
        const int64_t base = sptr[i >> 5] + 4 * (i & 31);
        const int64_t len = rp[i + 1] - rp[i];
        const int64_t wdt = (sptr[(i >> 5) + 1] - sptr[i >> 5]) / 32;
        for (int64_t k = 0; k < wdt; k++) {
          int loc = (int)(i - a);
          if (k < len) {
            const int j = cols[rp[i] + k];
            loc = (j >= a && j < b)
                      ? (int)(j - a)
                      : kTileNodes + hslot[std::lower_bound(hl.begin(), hl.end(), j) - hl.begin()];
          }
          lidx[base + (k >> 2) * 128 + (k & 3)] = (uint16_t)loc;
          if (boff_too) boff[base + (k >> 2) * 128 + (k & 3)] = (uint16_t)(16 * loc);
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < nthr; w++) pool.emplace_back(work, w);
  for (auto &th : pool) th.join();
  if (too_big[0]) return NLM_OK;
  // id block of a tile: its 8 slices, contiguous in the sliced layout
  int64_t ids_max = 0;
  for (int64_t t = 0; t < nt; t++) {
    const int64_t s0 = 8 * t, s1 = std::min<int64_t>(8 * t + 8, in.nslices);
    ids_max = std::max(ids_max, 2 * (sptr[s1] - sptr[s0]));
  }
  if (boff_too && ids_max > kTileIdsMaxBytes) return NLM_OK;
  if (in.lres)
    for (int64_t t = 0; t < nt; t++) halo[t] = std::move(halo_slots[t]);
  // Every tile's halo list is padded with empty slots (-1) to the longest,
  // so tile t's list starts at t x stride: a kernel finds it without a
  // dependent load of per-tile offsets.
  size_t nmax = 0;
  for (int64_t t = 0; t < nt; t++) nmax = std::max(nmax, halo[t].size());
  if ((int64_t)nmax * nt > (int64_t)INT32_MAX) return NLM_OK;
  std::vector<int> hall(std::max<int64_t>(1, (int64_t)nmax * nt), -1);
  for (int64_t t = 0; t < nt; t++)
    std::copy(halo[t].begin(), halo[t].end(), hall.begin() + t * (int64_t)nmax);
  uint16_t *d_l = nullptr;
  int *d_h = nullptr;
  NLM_CUDA(h->alloc(&d_l, lidx.size()));
  NLM_CUDA(h->alloc(&d_h, hall.size()));
  NLM_CUDA(cudaMemcpyAsync(d_l, lidx.data(), sizeof(uint16_t) * lidx.size(), cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaMemcpyAsync(d_h, hall.data(), sizeof(int) * hall.size(), cudaMemcpyHostToDevice, h->stream));
  uint8_t *d_r = nullptr;
  if (rint_too) {
    NLM_CUDA(h->alloc(&d_r, rint.size()));
    NLM_CUDA(cudaMemcpyAsync(d_r, rint.data(), rint.size(), cudaMemcpyHostToDevice, h->stream));
  }
  uint16_t *d_b = nullptr;
  if (boff_too) {
    NLM_CUDA(h->alloc(&d_b, boff.size()));
    NLM_CUDA(cudaMemcpyAsync(d_b, boff.data(), sizeof(uint16_t) * boff.size(),
                             cudaMemcpyHostToDevice, h->stream));
  }
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  h->D.tile_lidx = d_l;
  h->D.tile_boff = d_b;
  h->D.row_int = d_r;
  h->D.tile_ids_bytes = (int)ids_max;
  h->D.tile_halo = d_h;
  h->D.tile_nmax = kTileNodes + (int)nmax;
  h->D.tile_hstride = (int)nmax;
  ok = true;
  if (need_out) *need_out = std::move(need);
  return NLM_OK;
}

}  // namespace nlm
