// Rank-trimmed packing of a list of tiles: the device side of a TilePacker transfer
// (include/hcorepp/operators/interface/TilePacker.hpp:18-62 packs one tile at its full capacity,
// rows x max_rank + max_rank x cols; here a whole list is packed at once and a compressed tile
// contributes only the columns its rank uses).
//
// Packed format, tiles in list order, each starting at offsets[t] (doubles):
//   dense:           rows x cols, column-major
//   compressed:      U (rows x rank, ld rows) followed by V (rank x cols, ld rank)
//   compressed_vt:   U (rows x rank, ld rows) followed by W = V^T (cols x rank, ld cols)
// In the tile buffers both factor blocks are contiguous (U's leading dimension is rows, the V
// region's is rank for compressed and cols for compressed_vt), so every tile is at most two
// contiguous copies.  offsets[count] is the total.
#include "internal.cuh"

namespace hcgb {

namespace {

__device__ __forceinline__ long long packed_doubles(const DevTile &t) {
    if (!t.kind) return (long long) t.rows * t.cols;
    const long long r = *t.rank;
    return r * (t.rows + t.cols);
}

// offsets[0..n] = exclusive prefix sum of the packed sizes; one CTA: every thread sums a
// contiguous run of tiles, a Hillis-Steele scan combines the runs.
__global__ void __launch_bounds__(1024) pack_offsets_kernel(const DevTile *tiles, int n, long long *offsets) {
    __shared__ long long part[1024];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    const int b1 = b0 + per < n ? b0 + per : n;
    long long s = 0;
    for (int i = b0; i < b1; i++) s += packed_doubles(tiles[i]);
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < (int) blockDim.x; o <<= 1) {
        const long long v = (int) threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (int i = b0; i < b1; i++) {
        offsets[i] = run;
        run += packed_doubles(tiles[i]);
    }
    if (threadIdx.x == blockDim.x - 1) offsets[n] = part[blockDim.x - 1];
}

__device__ __forceinline__ void copy_run(const double *src, double *dst, long long len) {
    for (long long e = threadIdx.x; e < len; e += blockDim.x) dst[e] = src[e];
}

// One CTA per tile: unpack = 0 copies the tile's used part into the packed buffer, 1 back.
__global__ void __launch_bounds__(256) pack_kernel(const DevTile *tiles, int n, const long long *offsets,
                                                   double *packed, int unpack) {
    const int t = blockIdx.x;
    if (t >= n) return;
    const DevTile d = tiles[t];
    double *p = packed + offsets[t];
    if (!d.kind) {
        const long long len = (long long) d.rows * d.cols;
        if (unpack) copy_run(p, d.data, len);
        else copy_run(d.data, p, len);
        return;
    }
    const long long r = *d.rank;
    const long long lu = r * d.rows, lv = r * d.cols;
    if (unpack) {
        copy_run(p, d.data, lu);
        copy_run(p + lu, d.v, lv);
    } else {
        copy_run(d.data, p, lu);
        copy_run(d.v, p + lu, lv);
    }
}

}  // namespace

void launch_pack(const DevTile *tiles, int n, long long *offsets, double *packed, bool unpack, cudaStream_t st) {
    { pack_offsets_kernel<<<1, 1024, 0, st>>>(tiles, n, offsets); note_launch(); }
    { pack_kernel<<<n, 256, 0, st>>>(tiles, n, offsets, packed, unpack ? 1 : 0); note_launch(); }
}

}  // namespace hcgb
