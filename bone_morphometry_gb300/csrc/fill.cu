// Tile-owned sphere fill (local_thickness.rs:169-202) for sm_103a.
//
// The reference paints every voxel of every ridge ball with an atomic max:
// sum over ridges of |ball| operations (~7e10 for a 512^3 marrow phase, where
// every voxel is covered ~500 times).  Here the work splits in two:
//
// Selected voxels: the output volume is cut into 32x64x16 tiles (32x32x16 for
// volumes below 3 * 2^24 voxels, 32x16x16 below 2^24), each owned by one CTA
// that paints its tile in shared memory.  The balls that reach a tile
// are visited in strictly descending r^2 (a counting sort by (tile, r^2
// rank)); the final value of a voxel is the r^2 of the first -- largest --
// ball that covers it, so per-row bitmasks of still-unpainted voxels let every
// later ball skip whatever is already decided.  Balls of equal r^2 paint the
// same value and run concurrently; a barrier separates consecutive r^2 groups.
// Each group is processed in rounds: a plane test per (ball, plane) against a
// range-OR table of the masks, then a pass that paints the chords of the
// planes that passed, each plane walked by a group of 1 to 8 threads.
//
// Non-selected voxels: a ball reaches one only on its sphere (its r^2 is the
// distance to the nearest non-selected voxel), so a per-ridge pass over the
// sphere's lattice points adds those with an atomic max.
//
// The result is the reference's max-of-balls map bit for bit.
//
// Pipeline (one phase):
//   ridge_tile_kernel  -> ridge records + occ[r2] flags
//   scan(occ)          -> rank_desc[r2] (0 = largest r2 present), rvals[rank]
//   bin_kernel<COUNT>  -> counts[tile * nR + rank]   (tiles the ball's box touches
//                          and the ball reaches)
//   scan(counts)       -> offsets
//   bin_kernel<SCATTER>-> entries[offset..] = ball centre (linear index)
//   tile_fill_kernel   -> u32 r^2 map of the selected voxels
//   site_kernel        -> non-selected voxels on each ridge sphere (atomic max)
#include "kernels.h"

namespace bm {

namespace {

__device__ __forceinline__ uint32_t isqrt_u32(uint32_t v) { return isqrt30(v); }  // floor sqrt, v < 2^30

__device__ __forceinline__ uint32_t csqrt_u32(uint32_t v) {
  const uint32_t f = isqrt_u32(v);
  return f * f == v ? f : f + 1;
}

// The same floor square root where v < 2^24 is known.
__device__ __forceinline__ uint32_t isqrt24(uint32_t v) { return isqrt_u32(v); }

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr long long kScanTile = kScanThreads * kScanItems;

// Exclusive scan of one 4096-element tile; writes the tile total to sums.
__global__ void __launch_bounds__(kScanThreads)
scan_tile_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, long long n,
                 uint32_t* __restrict__ sums) {
  __shared__ uint32_t wsum[32];
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0u;
    t += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = wsum[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    wsum[lane] = wi - w;  // exclusive warp offsets
    if (lane == 31) sums[blockIdx.x] = wi;
  }
  __syncthreads();
  uint32_t run = wsum[warp] + inc - t;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, long long n, const uint32_t* __restrict__ tile_offsets) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] += tile_offsets[i / kScanTile];
}

// occ[0..rmax+1] flags (occ[rmax+1] = 0) -> ascending exclusive scan in
// rank_desc (so rank_desc[rmax+1] = nR, never rewritten) -> rank_desc[r2] =
// descending rank of every r2 present, rvals[rank] = r2, info->nR.
__global__ void rank_finalize_kernel(const uint32_t* __restrict__ occ, uint32_t* __restrict__ rank_desc, uint32_t rmax,
                                     uint32_t* __restrict__ rvals, uint4* __restrict__ rgeo,
                                     FillInfo* __restrict__ info) {
  const uint32_t nR = rank_desc[rmax + 1];
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r <= (long long)rmax;
       r += (long long)gridDim.x * blockDim.x) {
    if (occ[r]) {
      const uint32_t rk = nR - 1u - rank_desc[r];
      const uint32_t R = (uint32_t)r;
      rank_desc[r] = rk;
      rvals[rk] = R;
      rgeo[rk] = make_uint4(R, csqrt_u32(R), isqrt_u32(R), 0u);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) info->nR = nR;
}

struct Geom {
  int ntx, nty, ntz;
  long long ntiles;
  int ty;  // rows of y per tile (32 or 64)
};


// One thread per ridge: every tile whose box the ball reaches (closest point of
// the tile within r^2 of the centre).  COUNT: counts[bin]++; else: place the
// centre at offsets[bin] + (--counts[bin]).
template <bool COUNT>
__global__ void __launch_bounds__(256)
bin_kernel(const uint2* __restrict__ ridges, const Counters* __restrict__ ctr, const uint32_t* __restrict__ rank_desc,
           FillInfo* info, Dims dm, VoxelDecoder vd, Geom g, uint32_t* __restrict__ counts,
           const uint32_t* __restrict__ offsets, uint32_t* __restrict__ entries) {
  const unsigned long long nr = ctr->ridges;
  const uint32_t nR = info->nR;
  unsigned long long touched = 0, steps = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)nr;
       i += (long long)gridDim.x * blockDim.x) {
    const uint2 rec = ridges[i];
    const uint32_t R = rec.y;
    int x, y, z;
    vd(rec.x, x, y, z);
    const int rad = (int)csqrt_u32(R);
    const uint32_t rank = rank_desc[R];
    steps += ((unsigned)rad * 402u + 1023u) >> 10;  // ceil(2 pi rad / 16): 2 pi / 16 ~ 402 / 1024
    const int tx0 = max(x - rad, 0) / kFillTX, tx1 = min(x + rad, dm.w - 1) / kFillTX;
    const int ty0 = max(y - rad, 0) / g.ty, ty1 = min(y + rad, dm.h - 1) / g.ty;
    const int tz0 = max(z - rad, 0) / kFillTZ, tz1 = min(z + rad, dm.d - 1) / kFillTZ;
    for (int tz = tz0; tz <= tz1; ++tz) {
      const int bz0 = tz * kFillTZ, bz1 = bz0 + kFillTZ - 1;
      const long long ddz = z < bz0 ? bz0 - z : (z > bz1 ? z - bz1 : 0);
      for (int ty = ty0; ty <= ty1; ++ty) {
        const int by0 = ty * g.ty, by1 = by0 + g.ty - 1;
        const long long ddy = y < by0 ? by0 - y : (y > by1 ? y - by1 : 0);
        const long long dyz = ddz * ddz + ddy * ddy;
        if (dyz > (long long)R) continue;
        for (int tx = tx0; tx <= tx1; ++tx) {
          const int bx0 = tx * kFillTX, bx1 = bx0 + kFillTX - 1;
          const long long ddx = x < bx0 ? bx0 - x : (x > bx1 ? x - bx1 : 0);
          if (dyz + ddx * ddx > (long long)R) continue;
          const long long tile = ((long long)tz * g.nty + ty) * g.ntx + tx;
          const long long bin = tile * nR + rank;
          if (COUNT) {
            atomicAdd(&counts[bin], 1u);
            ++touched;
          } else {
            const uint32_t k = atomicSub(&counts[bin], 1u) - 1u;
            entries[offsets[bin] + k] = rec.x;
          }
        }
      }
    }
  }
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      touched += __shfl_xor_sync(0xffffffffu, touched, o);
      steps += __shfl_xor_sync(0xffffffffu, steps, o);
    }
    if ((threadIdx.x & 31) == 0 && touched) atomicAdd(&info->total_entries, touched);
    if ((threadIdx.x & 31) == 0 && steps) atomicAdd(&info->site_steps, steps);
    if (blockIdx.x == 0 && threadIdx.x == 0) info->ridges = nr;
  }
}

constexpr int kFillThreads = 256;
constexpr int kFillWarps = kFillThreads / 32;

__device__ __forceinline__ uint32_t range_mask(int a, int b) {  // bits a..b, 0 <= a <= b <= 31
  return (0xffffffffu >> (31 - b)) & (0xffffffffu << a);
}

// Word of row (z, y) in the unpainted-voxel masks of a tile with TY rows per
// plane: rotated by 3z within the plane, so that threads reading the same y of
// consecutive planes (the planes of one ball) fall into different banks.
template <int TY>
__device__ __forceinline__ int urow(int z, int y) { return z * TY + ((y + 3 * z) & (TY - 1)); }

constexpr int kBinChunk = 256;    // bins whose offsets are staged in shared memory at a time
constexpr int kEntWin = 768;      // ball entries staged in shared memory at a time
constexpr int kRotLevels = 6;     // range-OR levels: spans 1, 2, 4, 8, 16, 32 rows (level 0 is usel itself);
                                  // two 32-row lookups cover a plane's 64 rows
constexpr int kRotEvery = 4;      // non-empty bins between rebuilds of the range-OR table

// The tile shape: 32 x TY x 16 voxels, TY = 16, 32 or 64 rows of y.  Taller
// tiles give fewer ball entries and plane tests per voxel, shorter ones more
// tiles (a small volume's fill is bound by its tiles' serial chains of r^2 bins).
template <int TY>
struct FillTile {
  static_assert(TY == 16 || TY == 32 || TY == 64, "16, 32 or 64 rows per tile");
  static constexpr int kRows = kFillTZ * TY;
  static constexpr int kRotStride = TY + 1;  // words per range-OR row: lanes on different planes hit different banks
  // (ball, plane) paint items per round: as many as 5 CTAs per SM leave room for
  static constexpr int kItems = TY == 64 ? 2048 : 4096;
  static constexpr int kRound = kItems / kFillTZ;  // balls tested per round (each yields at most kFillTZ items)
  static constexpr size_t kSmemWords = (size_t)kRows + kRows + (kBinChunk + 4) + kBinChunk + kEntWin +
                                       (kRotLevels - 1) * kFillTZ * kRotStride + kItems + 130;
};
// a paint item packs (window index << 16) | (rows - 1) << 10 | first row << 4 | plane
static_assert(kEntWin <= (1 << 16) && kFillTZ <= 16, "paint item encoding (and rows per tile <= 64)");

// rot[lv - 1][z][y] (rows of TY + 1 words) = OR of the unpainted-voxel masks
// of rows y .. y + 2^lv - 1 of plane z (rows past the tile edge count as
// empty), lv = 1 .. 5.  Built with shuffles, one plane per warp step; lane l
// holds row l (and l + 32 in 64-row tiles; lanes past a 16-row tile hold nothing).
template <int TY>
__device__ __forceinline__ void build_rot(const uint32_t* __restrict__ usel, uint32_t* __restrict__ rot, int warp,
                                          int lane, int nwarps) {
  constexpr int kStride = FillTile<TY>::kRotStride;
  for (int zz = warp; zz < kFillTZ; zz += nwarps) {
    if constexpr (TY == 64) {
      uint32_t v0 = usel[urow<TY>(zz, lane)], v1 = usel[urow<TY>(zz, lane + 32)];
#pragma unroll
      for (int lv = 1; lv < kRotLevels; ++lv) {
        const int s = 1 << (lv - 1);  // row y takes the previous level's rows y and y + s
        const uint32_t a = __shfl_sync(0xffffffffu, v0, (lane + s) & 31);
        const uint32_t b = __shfl_sync(0xffffffffu, v1, (lane + s) & 31);
        const bool lo = lane + s < 32;
        v0 |= lo ? a : b;
        v1 |= lo ? b : 0u;
        uint32_t* rr = rot + ((lv - 1) * kFillTZ + zz) * kStride;
        rr[lane] = v0;
        rr[lane + 32] = v1;
      }
    } else {
      uint32_t v = lane < TY ? usel[urow<TY>(zz, lane)] : 0u;
#pragma unroll
      for (int lv = 1; lv < kRotLevels; ++lv) {
        const uint32_t u = __shfl_down_sync(0xffffffffu, v, 1 << (lv - 1));
        v |= (lane + (1 << (lv - 1)) < 32) ? u : 0u;
        if (lane < TY) rot[((lv - 1) * kFillTZ + zz) * kStride + lane] = v;
      }
    }
  }
}

// One CTA per tile (32 x TY x 16 voxels) paints the tile's selected voxels.
// A painted voxel's r^2 goes straight to the map (each selected voxel is
// painted once: its bit in usel is cleared atomically first), and the voxels
// left unpainted get 0 at the end; without a per-voxel value array the CTA
// needs 30 KB (16 rows), 37 KB (32 rows) or 44 KB (64 rows) of shared memory,
// and 5 CTAs share an SM (48 registers).
// Shared memory:
//   sown : per row (z, y), the tile's selected voxels;
//   usel : per row (z, y), the selected voxels not yet painted;
//   boff / nzb : the tile's bin offsets and the list of non-empty bins for
//          the current chunk of bins;
//   ent  : a window of the tile's ball entries, decoded to tile-local
//          coordinates (10 bits each, biased by 512);
//   rot  : range-OR table of usel (build_rot);
//   item : the (ball, plane) pairs of the current round that need painting.
// Bins arrive largest r^2 first with a barrier between bins, so the first ball
// to reach a voxel carries its final value and later balls skip decided
// voxels.  A bin is processed in rounds of up to kRound balls, each in two
// phases.  Test: each warp takes two balls (one per half-warp); lane hl of a
// half tests plane zlo + hl of its ball -- the plane needs work only if some
// open row in the disk's y-range has an unpainted voxel inside the disk's
// widest chord (a stale range-OR table is a superset, so it never skips work)
// -- and appends the planes that pass to the item list.  Paint: a group of
// 1 to 8 threads per item (more when the round has few items) walks the
// disk's rows and paints each row's chord of unpainted voxels.  Balls of one
// bin have the same r^2, so the order of their items does not matter (two
// threads may write the same value).  Non-selected voxels are left 0 here;
// the site pass or the chain passes add the ones a sphere reaches.
template <int TY>
__global__ void __launch_bounds__(kFillThreads, 5)
tile_fill_kernel(const uint32_t* __restrict__ entries, const uint32_t* __restrict__ offsets,
                 const uint32_t* __restrict__ rvals, const uint4* __restrict__ rgeo, const FillInfo* __restrict__ info,
                 const uint32_t* __restrict__ selbits, Dims dm, VoxelDecoder vd, Geom g,
                 const uint32_t* __restrict__ order, uint32_t* __restrict__ fillmap) {
  constexpr int kRows = FillTile<TY>::kRows;
  constexpr int kRotStride = FillTile<TY>::kRotStride;
  constexpr int kItems = FillTile<TY>::kItems;
  constexpr int kRound = FillTile<TY>::kRound;
  extern __shared__ uint32_t smem[];
  uint32_t* sown = smem;                                     // kRows: the tile's selected voxels per row
  uint32_t* usel = smem + kRows;                             // kRows
  uint32_t* boff = usel + kRows;                             // kBinChunk + 1
  uint32_t* nzb = boff + kBinChunk + 4;                      // kBinChunk
  uint32_t* ent = nzb + kBinChunk;                           // kEntWin
  uint32_t* rot = ent + kEntWin;                             // (kRotLevels - 1) * kFillTZ * kRotStride
  uint32_t* item = rot + (kRotLevels - 1) * kFillTZ * kRotStride;  // kItems
  uint16_t* hyt = reinterpret_cast<uint16_t*>(item + kItems);              // 257 (+1) half-words
  __shared__ uint32_t s_nnz, s_wlo, s_whi;
  __shared__ uint32_t s_nitem[2];
  __shared__ uint32_t wcnt[kFillWarps];
  __shared__ uint2 sgeo[kBinChunk];  // (r2, isqrt(r2)) of the chunk's non-empty bins
  const uint32_t nR = info->nR;
  const int nw = dm.nw();
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int hl = lane & 15, half = lane >> 4;
  const unsigned lanes_below = (1u << lane) - 1u;
  uint32_t parity = 0;  // which item counter the next round uses
  for (long long k = blockIdx.x; k < g.ntiles; k += gridDim.x) {
    const long long tile = order[k];  // heaviest tiles first
    const int tx = (int)(tile % g.ntx);
    const int ty = (int)((tile / g.ntx) % g.nty);
    const int tz = (int)(tile / ((long long)g.ntx * g.nty));
    const int x0 = tx * kFillTX, y0 = ty * TY, z0 = tz * kFillTZ;
    const int vx = min(kFillTX, dm.w - x0), vy = min(TY, dm.h - y0), vz = min(kFillTZ, dm.d - z0);
    const uint32_t xmask = vx >= 32 ? 0xffffffffu : ((1u << vx) - 1u);
    const uint32_t* off = offsets + tile * (long long)nR;
    if (off[0] == off[nR]) {  // no ball reaches this tile: all zero
      for (int r = warp; r < kRows; r += kFillWarps) {
        const int zz = r / TY, yy = r % TY;
        if (zz < vz && yy < vy && lane < vx)
          fillmap[((long long)(z0 + zz) * dm.h + (y0 + yy)) * dm.w + x0 + lane] = 0u;
      }
      continue;
    }
    if (tid == 0) {
      s_wlo = 0u;
      s_whi = 0u;
      s_nitem[0] = 0u;
      s_nitem[1] = 0u;
    }
    parity = 0;
    bool any_sel = false;
    for (int r = tid; r < kRows; r += kFillThreads) {
      const int zz = r / TY, yy = r % TY;
      uint32_t own = 0u;
      if (zz < vz && yy < vy) own = selbits[((long long)(z0 + zz) * dm.h + (y0 + yy)) * nw + tx] & xmask;
      usel[urow<TY>(zz, yy)] = own;
      sown[urow<TY>(zz, yy)] = own;
      any_sel = any_sel || own != 0u;
    }
    if (!__syncthreads_or(any_sel)) {  // nothing selected here (outside the ROI, say): all zero
      for (int r = warp; r < kRows; r += kFillWarps) {
        const int zz = r / TY, yy = r % TY;
        if (zz < vz && yy < vy && lane < vx)
          fillmap[((long long)(z0 + zz) * dm.h + (y0 + yy)) * dm.w + x0 + lane] = 0u;
      }
      continue;
    }
    build_rot<TY>(usel, rot, warp, lane, kFillWarps);
    for (uint32_t b0 = 0; b0 < nR; b0 += kBinChunk) {
      const uint32_t nb = min((uint32_t)kBinChunk, nR - b0);
      __syncthreads();
      for (uint32_t i = tid; i <= nb; i += kFillThreads) boff[i] = off[b0 + i];
      if (tid == 0) s_nnz = 0u;
      __syncthreads();
      // compact the non-empty bins, preserving order (warp ballots + one atomic per warp)
      for (uint32_t base = 0; base < nb; base += kFillThreads) {
        const uint32_t i = base + tid;
        const bool ne = i < nb && boff[i] != boff[i + 1];
        const unsigned m = __ballot_sync(0xffffffffu, ne);
        if (lane == 0) wcnt[warp] = __popc(m);
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += wcnt[w];
        if (ne) nzb[s_nnz + before + __popc(m & lanes_below)] = i;
        __syncthreads();
        if (tid == 0) {
          uint32_t t = 0;
          for (int w = 0; w < kFillWarps; ++w) t += wcnt[w];
          s_nnz += t;
        }
        __syncthreads();
      }
      const uint32_t nnz = s_nnz;
      for (uint32_t i = tid; i < nnz; i += kFillThreads) {
        const uint4 q = rgeo[b0 + nzb[i]];
        sgeo[i] = make_uint2(q.x, q.z);
      }
      __syncthreads();
      for (uint32_t k = 0; k < nnz; ++k) {
        const uint32_t bl = nzb[k];
        const uint2 gq = sgeo[k];
        const int R = (int)gq.x;
        const int rad = (int)gq.y;                         // isqrt(r2): no lattice point of the ball is further
        const uint32_t e = boff[bl + 1];
        // this bin's disk radii: hyt[|dz|] = isqrt(r2 - dz^2)
        for (int i = tid; i <= rad; i += kFillThreads) hyt[i] = (uint16_t)isqrt24((uint32_t)(R - i * i));
        if (k % kRotEvery == 0 && k > 0) build_rot<TY>(usel, rot, warp, lane, kFillWarps);
        __syncthreads();
        for (uint32_t ss = boff[bl]; ss < e;) {
          if (ss < s_wlo || ss >= s_whi) {  // reload the entry window at ss (uniform decision)
            __syncthreads();
            const uint32_t lo = ss, hi = min(ss + (uint32_t)kEntWin, off[nR]);
            for (uint32_t i = lo + tid; i < hi; i += kFillThreads) {
              int cx, cy, cz;
              vd(entries[i], cx, cy, cz);
              ent[i - lo] = (uint32_t)(cx - x0 + 512) | ((uint32_t)(cy - y0 + 512) << 10) |
                            ((uint32_t)(cz - z0 + 512) << 20);
            }
            if (tid == 0) {
              s_wlo = lo;
              s_whi = hi;
            }
            __syncthreads();
          }
          const uint32_t se = min(min(e, s_whi), ss + (uint32_t)kRound);
          const uint32_t wb = ss - s_wlo;  // window index of the round's first ball
          // test: two balls per warp step, one per half-warp (lanes 0..15 on
          // ball 2w, lanes 16..31 on 2w+1); lane hl tests plane zlo + hl of its
          // ball.  Two balls per step spread a round's balls over all warps
          // (four per step measured 2% slower: the last steps left warps idle).
          auto plane_test = [&](uint32_t bi, int& pya, int& pyb, int& zz) -> bool {
            const bool have = bi < se - ss;
            const uint32_t c = ent[wb + (have ? bi : 0u)];
            const int cx = (int)(c & 0x3ffu) - 512, cy = (int)((c >> 10) & 0x3ffu) - 512, cz = (int)(c >> 20) - 512;
            const int zlo = max(cz - rad, 0), zhi = min(cz + rad, vz - 1);
            zz = zlo + hl;
            const int dz = zz - cz;
            bool ok = have && zz <= zhi;  // then |dz| <= rad
            const int hy = (int)hyt[min(abs(dz), rad)];
            pya = max(cy - hy, 0);
            pyb = min(cy + hy, vy - 1);
            const int xa = max(cx - hy, 0), xb = min(cx + hy, vx - 1);
            ok = ok && pya <= pyb && xa <= xb;
            const int zc = min(zz, kFillTZ - 1);
            const int ya = min(pya, TY - 1), yb = max(min(pyb, TY - 1), ya);
            const int lv = min(31 - __clz(yb - ya + 1), kRotLevels - 1);  // 2^lv <= span: two lookups cover it
            const uint32_t* tl = rot + (max(lv - 1, 0) * kFillTZ + zc) * kRotStride;
            const uint32_t orr = lv == 0 ? usel[urow<TY>(zc, ya)] : (tl[ya] | tl[yb - (1 << lv) + 1]);
            return ok && (orr & range_mask(min(max(xa, 0), 31), max(min(xb, 31), min(max(xa, 0), 31)))) != 0u;
          };
          // items: (window index, rows ya .. ya + n, plane)
          auto append = [&](uint32_t bi, bool pass, int pya, int pyb, int zz) {
            const unsigned act = __ballot_sync(0xffffffffu, pass);
            if (act) {
              uint32_t base = 0;
              if (lane == 0) base = atomicAdd(&s_nitem[parity], (uint32_t)__popc(act));
              base = __shfl_sync(0xffffffffu, base, 0);
              if (pass)
                item[base + __popc(act & lanes_below)] =
                    ((wb + bi) << 16) | ((uint32_t)(pyb - pya) << 10) | ((uint32_t)pya << 4) | (uint32_t)zz;
            }
          };
          for (uint32_t bp = 2 * warp; bp < se - ss; bp += 2 * kFillWarps) {
            const uint32_t b1 = bp + half;
            int ya1, yb1, z1;
            const bool p1 = plane_test(b1, ya1, yb1, z1);
            append(b1, p1, ya1, yb1, z1);
          }
          __syncthreads();
          // paint: G threads per item (G = 1 .. 8, about twice as many as keep
          // the CTA's threads busy), each walking every G-th row of the plane's disk
          // and painting the row's chord of still-unpainted voxels.  Most
          // items that passed the range-OR test find nothing in any row.
          const uint32_t nitem = s_nitem[parity];
          if (tid == 0) s_nitem[parity ^ 1u] = 0u;  // the next round's counter (idle since the last barrier)
          const int lg = nitem >= 2 * kFillThreads ? 0 : nitem >= kFillThreads ? 1 : nitem >= kFillThreads / 2 ? 2 : 3;
          const int G = 1 << lg, sub = tid & (G - 1);
          for (uint32_t it = (uint32_t)(tid >> lg); it < nitem; it += (uint32_t)(kFillThreads >> lg)) {
            const uint32_t q = item[it];
            const int zz = (int)(q & 15u), ya = (int)((q >> 4) & 63u), yb = ya + (int)((q >> 10) & 63u);
            const uint32_t cb = ent[q >> 16];
            const int bx = (int)(cb & 0x3ffu) - 512, by = (int)((cb >> 10) & 0x3ffu) - 512;
            const int dz = zz - ((int)(cb >> 20) - 512);
            const int rz = R - dz * dz;
            // rows whose unpainted voxels all lie outside the disk's widest chord are skipped
            // before the row's own chord is computed
            const int hw = (int)hyt[abs(dz)];
            const uint32_t wide = range_mask(max(bx - hw, 0), min(bx + hw, vx - 1));
            for (int y = ya + sub; y <= yb; y += G) {
              const int row = urow<TY>(zz, y);
              const uint32_t m = usel[row] & wide;
              if (!m) continue;
              const int dy = y - by;
              const int t = rz - dy * dy;
              if (t < 0) continue;
              const int hx = (int)isqrt24((uint32_t)t);
              const int xa = max(bx - hx, 0), xb = min(bx + hx, vx - 1);
              if (xa > xb) continue;
              uint32_t bits = m & range_mask(xa, xb);
              if (!bits) continue;
              atomicAnd(&usel[row], ~bits);
              // every selected voxel is painted once (its bit cleared above): straight to the map
              uint32_t* orow = fillmap + ((long long)(z0 + zz) * dm.h + (y0 + y)) * dm.w + x0;
              while (bits) {
                orow[__ffs(bits) - 1] = (uint32_t)R;
                bits &= bits - 1u;
              }
            }
          }
          parity ^= 1u;
          __syncthreads();
          ss = se;
        }
      }
    }
    __syncthreads();
    // the voxels no ball painted (non-selected ones; the site pass adds those
    // a sphere reaches) get 0: one row per warp step
    for (int r = warp; r < kRows; r += kFillWarps) {
      const int zz = r / TY, yy = r % TY;
      const uint32_t painted = sown[urow<TY>(zz, yy)] & ~usel[urow<TY>(zz, yy)];
      if (zz < vz && yy < vy && lane < vx && !((painted >> lane) & 1u))
        fillmap[((long long)(z0 + zz) * dm.h + (y0 + yy)) * dm.w + x0 + lane] = 0u;
    }
    __syncthreads();
  }
}

// The non-selected voxels a ridge ball reaches.  A ball centred on p has r^2 =
// d^2(p), the squared distance from p to its nearest non-selected voxel, so the
// non-selected voxels inside it are exactly the non-selected lattice points of
// its sphere |v - p|^2 = r^2.  G lanes per ridge (16, or 8 when the spheres
// are small), lanes over the sphere's points; the map keeps the max over
// balls.  Runs after the tile fill, which leaves every non-selected voxel at 0.
template <int G>
__global__ void __launch_bounds__(256)
site_kernel(const uint2* __restrict__ ridges, const Counters* __restrict__ ctr, const uint32_t* __restrict__ selbits,
            const uint32_t* __restrict__ surf_off, const uint32_t* __restrict__ surf_pts, Dims dm, VoxelDecoder vd,
            uint32_t* __restrict__ fillmap) {
  constexpr int kLog = G == 16 ? 4 : 3;
  static_assert(G == (1 << kLog), "8 or 16 lanes per ridge");
  const unsigned long long nr = ctr->ridges;
  const int hl = threadIdx.x & (G - 1);
  const int nw = dm.nw();
  const long long hw0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> kLog;
  const long long nhw = ((long long)gridDim.x * blockDim.x) >> kLog;
  for (long long i = hw0; i < (long long)nr; i += nhw) {
    const uint2 rec = ridges[i];
    const uint32_t R = rec.y;
    int x, y, z;
    vd(rec.x, x, y, z);
    const uint32_t p1 = surf_off[R + 1];
    for (uint32_t p = surf_off[R] + hl; p < p1; p += G) {
      const uint32_t pk = surf_pts[p];
      const int sx = x + ((int)(pk << 22) >> 22);
      const int sy = y + ((int)(pk << 12) >> 22);
      const int sz = z + ((int)(pk << 2) >> 22);
      if ((unsigned)sx >= (unsigned)dm.w || (unsigned)sy >= (unsigned)dm.h || (unsigned)sz >= (unsigned)dm.d) continue;
      const uint32_t wbits = selbits[((long long)sz * dm.h + sy) * nw + (sx >> 5)];
      if ((wbits >> (sx & 31)) & 1u) continue;  // selected: painted by the tile fill
      uint32_t* dst = fillmap + ((long long)sz * dm.h + sy) * dm.w + sx;
      if (*dst < R) atomicMax(dst, R);
    }
  }
}

// Lattice points of the sphere |d|^2 = r2: one warp per r2.  COUNT:
// surf_cnt[r2] = number of points.  Else write them packed (10-bit two's
// complement dx | dy << 10 | dz << 20) from surf_off[r2] on.
template <bool COUNT>
__global__ void __launch_bounds__(256)
surf_kernel(uint32_t lo, uint32_t hi, uint32_t* __restrict__ surf_cnt, const uint32_t* __restrict__ surf_off,
            uint32_t* __restrict__ surf_pts) {
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long rr = (long long)lo + wid; rr <= (long long)hi; rr += nwarps) {
    const uint32_t R = (uint32_t)rr;
    const int r = (int)isqrt_u32(R);
    uint32_t total = 0;
    uint32_t pos0 = COUNT ? 0u : surf_off[R];
    for (int c0 = -r; c0 <= r; c0 += 32) {
      const int dz = c0 + lane;
      uint32_t mine = 0;
      if (dz <= r) {
        const uint32_t rz = R - (uint32_t)(dz * dz);
        const int ry = (int)isqrt_u32(rz);
        for (int dy = -ry; dy <= ry; ++dy) {
          const uint32_t rx2 = rz - (uint32_t)(dy * dy);
          const uint32_t k = isqrt_u32(rx2);
          if (k * k == rx2) mine += k ? 2u : 1u;
        }
      }
      uint32_t incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
      }
      if (!COUNT && dz <= r) {
        uint32_t pos = pos0 + incl - mine;
        const uint32_t rz = R - (uint32_t)(dz * dz);
        const int ry = (int)isqrt_u32(rz);
        for (int dy = -ry; dy <= ry; ++dy) {
          const uint32_t rx2 = rz - (uint32_t)(dy * dy);
          const uint32_t k = isqrt_u32(rx2);
          if (k * k != rx2) continue;
          const uint32_t yz = (((uint32_t)dy & 0x3ffu) << 10) | (((uint32_t)dz & 0x3ffu) << 20);
          surf_pts[pos++] = (k & 0x3ffu) | yz;
          if (k) surf_pts[pos++] = ((uint32_t)(-(int)k) & 0x3ffu) | yz;
        }
      }
      const uint32_t chunk = __shfl_sync(0xffffffffu, incl, 31);
      pos0 += chunk;
      total += chunk;
    }
    if (COUNT && lane == 0) surf_cnt[R] = total;
  }
}

Geom geom_of(Dims dm, int ty) {
  Geom g;
  g.ty = ty;
  g.ntx = (dm.w + kFillTX - 1) / kFillTX;
  g.nty = (dm.h + ty - 1) / ty;
  g.ntz = (dm.d + kFillTZ - 1) / kFillTZ;
  g.ntiles = (long long)g.ntx * g.nty * g.ntz;
  return g;
}

inline unsigned blocks_for(long long work, int per_block, long long cap) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

}  // namespace

int fill_tile_rows(Dims dm, int requested) {
  if (requested == 16 || requested == 32 || requested == 64) return requested;
  return dm.n() >= kFillTallMinVoxels ? 64 : dm.n() >= kFillMidMinVoxels ? 32 : 16;
}

long long fill_tile_count(Dims dm, int ty) { return geom_of(dm, ty).ntiles; }

size_t scan_scratch_words(long long n) {
  size_t words = 0;
  while (n > 1) {
    n = (n + kScanTile - 1) / kScanTile;
    words += (size_t)n + 1;
  }
  return words + 1;
}

cudaError_t launch_scan(const uint32_t* in, uint32_t* out, long long n, uint32_t* scratch, cudaStream_t s,
                        unsigned long long* launches) {
  if (n <= 0) return cudaSuccess;
  const long long nb = (n + kScanTile - 1) / kScanTile;
  uint32_t* sums = scratch;
  scan_tile_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, sums);
  ++*launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nb == 1) return e;
  e = launch_scan(sums, sums, nb, scratch + nb + 1, s, launches);
  if (e != cudaSuccess) return e;
  scan_add_kernel<<<blocks_for(n, 256, 152 * 64), 256, 0, s>>>(out, n, sums);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_rank(const uint32_t* occ, uint32_t* rank_desc, uint32_t rmax, uint32_t* rvals, uint4* rgeo,
                        FillInfo* info, uint32_t* scan_scratch, cudaStream_t s, unsigned long long* launches) {
  cudaError_t e = launch_scan(occ, rank_desc, (long long)rmax + 2, scan_scratch, s, launches);
  if (e != cudaSuccess) return e;
  rank_finalize_kernel<<<blocks_for((long long)rmax + 1, 256, 1024), 256, 0, s>>>(occ, rank_desc, rmax, rvals, rgeo,
                                                                                  info);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_bin(bool count, const uint2* ridges, const Counters* ctr, unsigned long long max_ridges,
                       const uint32_t* rank_desc, FillInfo* info, Dims dm, int ty, uint32_t* counts,
                       const uint32_t* offsets, uint32_t* entries, cudaStream_t s, unsigned long long* launches) {
  const Geom g = geom_of(dm, ty);
  const unsigned blocks = blocks_for((long long)max_ridges, 256, 152 * 32);
  if (count)
    bin_kernel<true><<<blocks, 256, 0, s>>>(ridges, ctr, rank_desc, info, dm, VoxelDecoder::of(dm), g, counts,
                                            offsets, entries);
  else
    bin_kernel<false><<<blocks, 256, 0, s>>>(ridges, ctr, rank_desc, info, dm, VoxelDecoder::of(dm), g, counts,
                                             offsets, entries);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_surf(bool count, uint32_t lo, uint32_t hi, uint32_t* surf_cnt, const uint32_t* surf_off,
                        uint32_t* surf_pts, cudaStream_t s, unsigned long long* launches) {
  if (hi < lo) return cudaSuccess;
  const unsigned blocks = blocks_for((long long)hi - lo + 1, 8, 152 * 16);
  if (count)
    surf_kernel<true><<<blocks, 256, 0, s>>>(lo, hi, surf_cnt, surf_off, surf_pts);
  else
    surf_kernel<false><<<blocks, 256, 0, s>>>(lo, hi, surf_cnt, surf_off, surf_pts);
  ++*launches;
  return cudaGetLastError();
}

namespace {

// Tile order of the fill: heaviest first (largest-processing-time order), so
// that the last CTAs to start are short ones and the launch has no long
// tail.  A tile's weight is its ball-entry count; tiles are counting-sorted
// into buckets of a quarter octave of that count, descending.
constexpr int kOrderBuckets = 132;

__device__ __forceinline__ int weight_bucket(uint32_t c) {
  if (c == 0u) return 0;
  const int b = 1 + (int)(4.0f * __log2f((float)c));
  return b < kOrderBuckets - 1 ? b : kOrderBuckets - 1;
}

__device__ __forceinline__ uint32_t tile_entries(const uint32_t* offsets, uint32_t nR, long long t) {
  return offsets[(t + 1) * (long long)nR] - offsets[t * (long long)nR];
}

__global__ void tile_weight_hist_kernel(const uint32_t* __restrict__ offsets, const FillInfo* __restrict__ info,
                                        long long ntiles, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kOrderBuckets];
  for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  const uint32_t nR = info->nR;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += (long long)gridDim.x * blockDim.x)
    atomicAdd(&h[weight_bucket(tile_entries(offsets, nR, t))], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

// hist -> start of every bucket in descending bucket order (one thread).
__global__ void tile_weight_scan_kernel(uint32_t* __restrict__ hist) {
  uint32_t run = 0;
  for (int b = kOrderBuckets - 1; b >= 0; --b) {
    const uint32_t c = hist[b];
    hist[b] = run;
    run += c;
  }
}

__global__ void tile_weight_scatter_kernel(const uint32_t* __restrict__ offsets, const FillInfo* __restrict__ info,
                                           long long ntiles, uint32_t* __restrict__ start,
                                           uint32_t* __restrict__ order) {
  const uint32_t nR = info->nR;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += (long long)gridDim.x * blockDim.x)
    order[atomicAdd(&start[weight_bucket(tile_entries(offsets, nR, t))], 1u)] = (uint32_t)t;
}

}  // namespace

size_t tile_order_words(Dims dm, int ty) { return (size_t)geom_of(dm, ty).ntiles + kOrderBuckets; }

namespace {
template <int TY>
cudaError_t launch_tile_fill_rows(const uint32_t* entries, const uint32_t* offsets, const uint32_t* rvals,
                                  const uint4* rgeo, const FillInfo* info, const uint32_t* selbits, Dims dm,
                                  const Geom& g, const uint32_t* order, uint32_t* fillmap, cudaStream_t s) {
  const size_t smem = FillTile<TY>::kSmemWords * sizeof(uint32_t);
  cudaError_t e = cudaFuncSetAttribute(tile_fill_kernel<TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long grid = g.ntiles < (1LL << 31) - 1 ? g.ntiles : (1LL << 31) - 1;
  tile_fill_kernel<TY><<<(unsigned)grid, kFillThreads, smem, s>>>(entries, offsets, rvals, rgeo, info, selbits, dm,
                                                                   VoxelDecoder::of(dm), g, order, fillmap);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_tile_fill(const uint32_t* entries, const uint32_t* offsets, const uint32_t* rvals,
                             const uint4* rgeo, const FillInfo* info, const uint32_t* selbits, Dims dm, int ty,
                             uint32_t* order_scratch, uint32_t* fillmap, cudaStream_t s, unsigned long long* launches) {
  const Geom g = geom_of(dm, ty);
  cudaError_t e;
  uint32_t* hist = order_scratch;
  uint32_t* order = order_scratch + kOrderBuckets;
  e = cudaMemsetAsync(hist, 0, kOrderBuckets * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const unsigned ob = blocks_for(g.ntiles, 256, 152 * 4);
  tile_weight_hist_kernel<<<ob, 256, 0, s>>>(offsets, info, g.ntiles, hist);
  tile_weight_scan_kernel<<<1, 1, 0, s>>>(hist);
  tile_weight_scatter_kernel<<<ob, 256, 0, s>>>(offsets, info, g.ntiles, hist, order);
  e = ty == 64   ? launch_tile_fill_rows<64>(entries, offsets, rvals, rgeo, info, selbits, dm, g, order, fillmap, s)
      : ty == 32 ? launch_tile_fill_rows<32>(entries, offsets, rvals, rgeo, info, selbits, dm, g, order, fillmap, s)
                 : launch_tile_fill_rows<16>(entries, offsets, rvals, rgeo, info, selbits, dm, g, order, fillmap, s);
  *launches += 4;
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_sites(const uint2* ridges, const Counters* ctr, unsigned long long max_ridges,
                         const uint32_t* selbits, const uint32_t* surf_off, const uint32_t* surf_pts, bool small,
                         Dims dm, uint32_t* fillmap, cudaStream_t s, unsigned long long* launches) {
  const unsigned blocks = blocks_for((long long)max_ridges, small ? 32 : 16, 152 * 16);
  if (small)
    site_kernel<8><<<blocks, 256, 0, s>>>(ridges, ctr, selbits, surf_off, surf_pts, dm, VoxelDecoder::of(dm), fillmap);
  else
    site_kernel<16><<<blocks, 256, 0, s>>>(ridges, ctr, selbits, surf_off, surf_pts, dm, VoxelDecoder::of(dm), fillmap);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace bm
