// Site values of the sphere fill by reverse chain passes (local_thickness.rs:
// 169-202, the non-selected voxels a ridge ball reaches) for sm_103a.
//
// A ridge ball centred on c has r^2 = m(c), the squared distance to the
// nearest non-selected voxel, so the non-selected voxels it reaches are
// exactly c's nearest sites.  The separable EDT finds them as nested argmins:
//   m(x,y,z)  = min_z' g(x,y,z') + (z - z')^2      (z pass)
//   g(x,y,z') = min_y' f(x,y',z') + (y - y')^2     (y pass)
//   f(x,y',z') = (x - x')^2, x' the nearest sites of the row (x pass)
// and (x', y', z') is a nearest site of c iff z', y', x' each attain their
// minimum (a nested minimum is attained exactly where every level is).  So
// the max r^2 over the balls reaching a site is a max pushed backwards along
// every tied argmin: first along z (chain_z), then along y with the x step
// folded in (chain_y).  Every push is an equality test against the exact
// minimum, so the result is the max-of-balls value of the reference bit for
// bit, whatever the ties.  The work is two window passes over the volume
// instead of one test per lattice point of every ridge sphere.
//
// Geometry (both passes): a CTA owns 32 consecutive x of one line-row and
// kChainTL consecutive outputs along the axis, stages the pass input with a
// halo of H rows on each side (H > isqrt of every minimum pushed, so every
// argmin lies in the staged rows; every pushed minimum and value is below
// 2^11), accumulates the pushed maxima per staged cell in shared memory and
// flushes the non-zero cells with global atomics.
#include "kernels.h"

namespace bm {

namespace {

constexpr int kChainTL = 128;
constexpr int kChainThreads = 256;
constexpr int kChainWarps = kChainThreads / 32;
constexpr int kChainPer = kChainTL / kChainWarps;  // outputs per thread (rows warp + 8 j)
constexpr int kChainRowsPerList = 4;                // rows of a warp compacted into one push list

// AXIS 2 (chain_z): lines along z at y = orow; in = g, outv = m, the pushed
// value is m at ridge voxels (bits = ridge bitmask); flush into dst = chain.
// AXIS 1 (chain_y): lines along y at z = orow; in = f, outv = g, the pushed
// value is chain (val); the flush takes the x step: the cell (x, y', z) with
// f = k^2 reaches the sites x - k and x + k of its row (bits = selection
// bitmask, a site is a 0 bit), max into dst = sites.
template <int AXIS>
__global__ void __launch_bounds__(kChainThreads, 4)
chain_kernel(const uint32_t* __restrict__ in, const uint32_t* __restrict__ outv, const uint32_t* __restrict__ val,
             const uint32_t* __restrict__ bits, uint32_t* __restrict__ dst, Dims dm, int n, long long stride,
             long long outer_stride, int nxt, int nchunk, int H) {
  extern __shared__ uint32_t sm[];
  const int rows = kChainTL + 2 * H;
  uint32_t* sin = sm;              // rows x 32: staged input (kInfSq outside the line)
  uint32_t* acc = sm + rows * 32;  // rows x 32: largest value pushed to the cell
  uint32_t* lst = acc + rows * 32;  // per warp: the push list (kChainRowsPerList * 32 entries)
  uint32_t* sel5 = lst + kChainWarps * kChainRowsPerList * 32;  // AXIS 1: rows x 5 selection words, x words
                                                                 // xt-2 .. xt+2 (the x step's sites)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long bid = blockIdx.x;
  const int xt = (int)(bid % nxt);
  const int chunk = (int)((bid / nxt) % nchunk);
  const int orow = (int)(bid / ((long long)nxt * nchunk));
  const int x = xt * 32 + lane;
  const bool xin = x < dm.w;
  const int nw = dm.nw();
  const long long base = (long long)orow * outer_stride + x;
  const int q0 = chunk * kChainTL;
  // the warp's outputs first (their loads in flight during the staging)
  uint32_t o[kChainPer], v[kChainPer];
#pragma unroll
  for (int j = 0; j < kChainPer; ++j) {
    const int q = q0 + warp + kChainWarps * j;
    const bool qin = xin && q < n;
    if (AXIS == 2) {  // only ridge voxels push: the others' minima are not read
      const uint32_t rb = q < n ? bits[((long long)q * dm.h + orow) * nw + xt] : 0u;  // one word per warp
      const bool ridge = qin && ((rb >> lane) & 1u);
      o[j] = ridge ? outv[base + (long long)q * stride] : 0u;
      v[j] = o[j];
    } else {  // only cells with a chain value push
      v[j] = qin ? val[base + (long long)q * stride] : 0u;
      o[j] = v[j] ? outv[base + (long long)q * stride] : 0u;
    }
  }
  // a block with nothing to push has nothing to flush either
  bool any = false;
#pragma unroll
  for (int j = 0; j < kChainPer; ++j) any = any || (v[j] != 0u && o[j] < kInfSq);
  if (!__syncthreads_or(any)) return;
  // staging: each warp's rows in batches whose loads are issued before the
  // shared-memory stores, so that their latencies overlap
  constexpr int kBatch = 6;
  for (int r0 = warp; r0 < rows; r0 += kChainWarps * kBatch) {
    uint32_t t[kBatch];
#pragma unroll
    for (int b = 0; b < kBatch; ++b) {
      const int r = r0 + kChainWarps * b, q = q0 - H + r;
      t[b] = (r < rows && xin && q >= 0 && q < n) ? in[base + (long long)q * stride] : kInfSq;
    }
#pragma unroll
    for (int b = 0; b < kBatch; ++b) {
      const int r = r0 + kChainWarps * b;
      if (r < rows) {
        sin[r * 32 + lane] = t[b];
        acc[r * 32 + lane] = 0u;
      }
    }
  }
  if (AXIS == 1) {
    // every site the x step can reach lies within kChainMaxHalo <= 64 of its
    // cell: words xt - 2 .. xt + 2 of the cell's row (1 = selected, no site)
    for (int k = threadIdx.x; k < rows * 5; k += kChainThreads) {
      const int r = k / 5, c = xt - 2 + k % 5, q = q0 - H + r;
      sel5[k] = (q >= 0 && q < n && c >= 0 && c < nw) ? bits[((long long)orow * dm.h + q) * nw + c] : ~0u;
    }
  }
  __syncthreads();
  // push: every p with in(p) + (q - p)^2 = outv(q) is an argmin of output q;
  // |q - p| <= isqrt(outv(q)) < H keeps p inside the staged rows.  The warp's
  // outputs that push are compacted (four rows at a time, 128 candidates) so
  // that every lane scans one whatever the ridge density; an entry packs row
  // j, column, minimum and value (both below 2^11: the caller's bound)
  uint32_t* wl = lst + warp * (kChainRowsPerList * 32);
  const unsigned lanes_below = (1u << lane) - 1u;
#pragma unroll
  for (int j0 = 0; j0 < kChainPer; j0 += kChainRowsPerList) {
    int cnt = 0;
#pragma unroll
    for (int jj = 0; jj < kChainRowsPerList; ++jj) {
      const int j = j0 + jj;
      const bool has = v[j] != 0u && o[j] < kInfSq;
      const unsigned m = __ballot_sync(0xffffffffu, has);
      if (has)
        wl[cnt + __popc(m & lanes_below)] =
            ((uint32_t)j << 27) | ((uint32_t)lane << 22) | (o[j] << 11) | v[j];
      cnt += __popc(m);
    }
    __syncwarp();
    for (int k = lane; k < cnt; k += 32) {
      const uint32_t e = wl[k];
      const int j = (int)(e >> 27), c = (int)((e >> 22) & 31u);
      const uint32_t oq = (e >> 11) & 2047u, vq = e & 2047u;
      const int i = H + warp + kChainWarps * j;
      const uint32_t* col = sin + i * 32 + c;
      uint32_t* ac = acc + i * 32 + c;
      if (col[0] == oq) atomicMax(ac, vq);
      for (int dp = 1; (uint32_t)(dp * dp) <= oq && dp < H; ++dp) {
        const uint32_t need = oq - (uint32_t)(dp * dp);
        if (col[-dp * 32] == need) atomicMax(ac - dp * 32, vq);
        if (col[dp * 32] == need) atomicMax(ac + dp * 32, vq);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  // flush the cells that received a value (the halo cells belong to the
  // neighbouring chunks, whose pushes meet them in the global max)
  for (int r = warp; r < rows; r += kChainWarps) {
    const int q = q0 - H + r;
    const uint32_t a = acc[r * 32 + lane];
    if (!a || !xin || q < 0 || q >= n) continue;
    if (AXIS == 2) {
      atomicMax(dst + base + (long long)q * stride, a);
    } else {
      const uint32_t f = sin[r * 32 + lane];  // (x - x')^2 for the nearest sites x' of row (q, orow)
      if (f >= kInfSq) continue;              // no site in the row: never an argmin (a guard)
      const int k = (int)isqrt30(f);  // k < H <= 64: the sites lie in the staged words
      uint32_t* drow = dst + ((long long)orow * dm.h + q) * dm.w;
      const uint32_t* sw = sel5 + r * 5 - (xt - 2);  // sw[word] for words xt-2 .. xt+2
      const int t1 = x - k, t2 = x + k;
      if (t1 >= 0 && !((sw[t1 >> 5] >> (t1 & 31)) & 1u)) atomicMax(drow + t1, a);
      if (k > 0 && t2 < dm.w && !((sw[t2 >> 5] >> (t2 & 31)) & 1u)) atomicMax(drow + t2, a);
    }
  }
}

template <int AXIS>
cudaError_t launch_chain(const uint32_t* in, const uint32_t* outv, const uint32_t* val, const uint32_t* bits,
                         uint32_t* dst, Dims dm, int halo, cudaStream_t s) {
  if (halo < 1 || halo > kChainMaxHalo) return cudaErrorInvalidValue;
  int n;
  long long stride, outer, orows;
  if (AXIS == 1) {
    n = dm.h;
    stride = dm.w;
    outer = (long long)dm.w * dm.h;
    orows = dm.d;
  } else {
    n = dm.d;
    stride = (long long)dm.w * dm.h;
    outer = dm.w;
    orows = dm.h;
  }
  const int nxt = (dm.w + 31) / 32;
  const int nchunk = (n + kChainTL - 1) / kChainTL;
  const long long blocks = (long long)nxt * nchunk * orows;
  const size_t smem = ((size_t)(2 * 32 + (AXIS == 1 ? 5 : 0)) * (kChainTL + 2 * halo) +
                       (size_t)kChainWarps * kChainRowsPerList * 32) * sizeof(uint32_t);
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(chain_kernel<AXIS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  chain_kernel<AXIS><<<(unsigned)blocks, kChainThreads, smem, s>>>(in, outv, val, bits, dst, dm, n, stride, outer, nxt,
                                                                   nchunk, halo);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_chain_z(const uint32_t* g, const uint32_t* m, const uint32_t* ridgebits, uint32_t* chain, Dims dm,
                           int halo, cudaStream_t s, unsigned long long* launches) {
  ++*launches;
  return launch_chain<2>(g, m, nullptr, ridgebits, chain, dm, halo, s);
}

cudaError_t launch_chain_y(const uint32_t* f, const uint32_t* g, const uint32_t* chain, const uint32_t* selbits,
                           uint32_t* sites, Dims dm, int halo, cudaStream_t s, unsigned long long* launches) {
  ++*launches;
  return launch_chain<1>(f, g, chain, selbits, sites, dm, halo, s);
}

}  // namespace bm
