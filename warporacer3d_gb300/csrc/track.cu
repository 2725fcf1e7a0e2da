// Track compilation on the GPU: the per-cell work of the reference's track
// compiler (racer/track.py:54-125) as CUDA kernels, in binary64 without
// contraction, so the packed grids equal the reference's bit for bit.
//
//   k_cells        racer/track.py:73-86, 89, 56  passes of the route over
//                  each cell (ball query of radius half_width + 0.5), the
//                  nearest waypoint of each pass, their reduction to layers,
//                  and the nearest waypoint overall
//   k_fill         racer/track.py:94-104         clearance, height, waypoint
//   k_ramps        racer/track.py:111-118        ramp boxes onto the heights
//   k_ft_columns,  racer/track.py:119-120        feature transform (nearest
//   k_ft_rows                                    road cell of every cell)
//   k_blur_*       racer/track.py:121            Gaussian blur, sigma 1.5
//   k_image_clear  racer/track.py:57             signed distance of an image
//
// Nearest-waypoint searches are exact brute force over a candidate list: a
// block of 16 x 16 cells keeps, in ascending index order, every waypoint
// whose distance to the block's bounding box could make it the nearest of
// some cell or put it inside the ball of one (bounds with a relative margin
// of 1e-9, far above the rounding of the distances), so each cell scans a
// few waypoints in the order the full scan would. Ties go to the lower
// index, as the reference's arrays show.
//
// The feature transform is the separable exact Euclidean method of Maurer,
// Qi and Raghavan (2003): per column the nearest feature row (ties to the
// lower row), then per row the lower envelope of those candidates (ties to
// the lower column). The blur is the 13-tap correlation of sigma 1.5 with
// reflected edges, axis 0 then axis 1, each output summed as its centre tap
// and then symmetric pairs from the outermost inward.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace {

constexpr int TILE = 16;  // cells per block edge in k_cells
constexpr int MAX_PASSES = 8;
constexpr int CAND_MAX = 2048;

struct RampRow {
  double cx, cy, c, s, length, width, height, rise;
};

struct Blur {
  double w[13];
};

struct CellArgs {
  const double* route;  // [W][3]
  int W;
  double x0, y0, cell;
  int nx, ny;
  double r2;             // ball radius squared; negative: nearest waypoint only
  int* nearest;          // [cells]
  int* count;            // [cells] layers kept (ball query only)
  int* pw;               // [cells][MAX_PASSES]
  unsigned char* upper;  // [W]
  int* error;
};

__device__ __forceinline__ double cell_x(double x0, double cell, int ix) { return x0 + cell * (double)ix; }

// One cell's nearest waypoint (*nearest) and, for a ball query, its passes
// and the nearest waypoint of each, over the candidates `cw` (indices,
// ascending) with coordinates `cxy` (racer/track.py:73-86 and 89).
__device__ int cell_passes(const CellArgs& a, const int* cw, const double2* cxy, int n, double x, double y,
                           int* out, int* nearest) {
  int pbest[MAX_PASSES];
  double pd[MAX_PASSES];
  int np = 0, first = -1, last = -10, best = 0;
  double bd2 = INFINITY;
  for (int i = 0; i < n; ++i) {
    const int w = cw ? cw[i] : i;
    const double2 r = cxy ? cxy[i] : make_double2(a.route[3 * w], a.route[3 * w + 1]);
    const double dx = r.x - x, dy = r.y - y;
    const double d2 = dx * dx + dy * dy;
    if (d2 < bd2) bd2 = d2, best = w;
    if (!(d2 <= a.r2)) continue;
    const double d = sqrt(d2);
    if (np == 0 || w - last > 2) {  // a gap of more than 2 starts a new pass
      if (np == MAX_PASSES) return -1;
      pbest[np] = w, pd[np] = d, ++np;
    } else if (d < pd[np - 1]) {
      pbest[np - 1] = w, pd[np - 1] = d;
    }
    if (first < 0) first = w;
    last = w;
  }
  *nearest = best;
  if (np == 0) return 0;
  if (np > 1 && first == 0 && last == a.W - 1) {  // the pass through the seam: its end, then its start
    int bw = pbest[np - 1];
    double bd = pd[np - 1];
    if (pd[0] < bd) bw = pbest[0], bd = pd[0];
    pbest[0] = bw, pd[0] = bd, --np;
  }
  for (int i = 1; i < np; ++i) {  // stable sort by height
    const int w = pbest[i];
    const double d = pd[i], z = a.route[3 * w + 2];
    int j = i;
    while (j > 0 && a.route[3 * pbest[j - 1] + 2] > z) pbest[j] = pbest[j - 1], pd[j] = pd[j - 1], --j;
    pbest[j] = w, pd[j] = d;
  }
  if (a.route[3 * pbest[np - 1] + 2] - a.route[3 * pbest[0] + 2] < 0.3) {  // one level: the nearest pass
    int bw = pbest[0];
    double bd = pd[0];
    for (int i = 1; i < np; ++i)
      if (pd[i] < bd) bw = pbest[i], bd = pd[i];
    out[0] = bw;
    return 1;
  }
  for (int i = 0; i < np; ++i) out[i] = pbest[i];
  return np;
}

__global__ void __launch_bounds__(TILE * TILE) k_cells(CellArgs a) {
  __shared__ double2 s_xy[CAND_MAX];
  __shared__ int s_w[CAND_MAX];
  __shared__ double s_min[TILE * TILE / 32];
  __shared__ int s_warp[TILE * TILE / 32];
  __shared__ int s_total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ix0 = blockIdx.x * TILE, iy0 = blockIdx.y * TILE;
  const double bx0 = cell_x(a.x0, a.cell, ix0), bx1 = cell_x(a.x0, a.cell, min(ix0 + TILE - 1, a.nx - 1));
  const double by0 = cell_x(a.y0, a.cell, iy0), by1 = cell_x(a.y0, a.cell, min(iy0 + TILE - 1, a.ny - 1));

  // the smallest, over waypoints, of the distance to the box's farthest point
  double m = INFINITY;
  for (int w = tid; w < a.W; w += blockDim.x) {
    const double rx = a.route[3 * w], ry = a.route[3 * w + 1];
    const double fx = fmax(fabs(rx - bx0), fabs(rx - bx1)), fy = fmax(fabs(ry - by0), fabs(ry - by1));
    m = fmin(m, fx * fx + fy * fy);
  }
  for (int o = 16; o; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) s_min[warp] = m;
  if (tid == 0) s_total = 0;
  __syncthreads();
  m = s_min[0];
  for (int i = 1; i < TILE * TILE / 32; ++i) m = fmin(m, s_min[i]);
  const double thr = fmax(m, a.r2) * (1.0 + 1e-9) + 1e-9;

  // candidates: waypoints whose distance to the box is within thr, in index order
  bool overflow = false;
  for (int base = 0; base < a.W; base += blockDim.x) {
    const int w = base + tid;
    bool take = false;
    double rx = 0.0, ry = 0.0;
    if (w < a.W) {
      rx = a.route[3 * w], ry = a.route[3 * w + 1];
      const double dx = fmax(fmax(bx0 - rx, rx - bx1), 0.0), dy = fmax(fmax(by0 - ry, ry - by1), 0.0);
      take = dx * dx + dy * dy <= thr;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, take);
    if (lane == 0) s_warp[warp] = __popc(ballot);
    __syncthreads();
    int offset = s_total;
    for (int i = 0; i < warp; ++i) offset += s_warp[i];
    offset += __popc(ballot & ((1u << lane) - 1u));
    if (take && offset < CAND_MAX) s_w[offset] = w, s_xy[offset] = make_double2(rx, ry);
    __syncthreads();
    if (tid == 0)
      for (int i = 0; i < TILE * TILE / 32; ++i) s_total += s_warp[i];
    __syncthreads();
  }
  const int total = s_total;
  overflow = total > CAND_MAX;  // scan every waypoint from global memory instead

  const int ix = ix0 + (tid % TILE), iy = iy0 + (tid / TILE);
  if (ix >= a.nx || iy >= a.ny) return;
  const double x = cell_x(a.x0, a.cell, ix), y = cell_x(a.y0, a.cell, iy);
  const long k = (long)iy * a.nx + ix;
  const int n = overflow ? a.W : total;
  const int* cw = overflow ? nullptr : s_w;
  const double2* cxy = overflow ? nullptr : s_xy;
  int out[MAX_PASSES], best = 0;
  const int got = cell_passes(a, cw, cxy, n, x, y, out, &best);
  a.nearest[k] = best;
  if (a.r2 < 0.0) return;
  if (got < 0) {
    atomicExch(a.error, 4);
    a.count[k] = 0;
    return;
  }
  a.count[k] = got;
  for (int i = 0; i < got; ++i) {
    a.pw[k * MAX_PASSES + i] = out[i];
    if (i > 0) a.upper[out[i]] = 1;
  }
}

// Bit 1: some pass lies on the lower layer; bit 2: some on the upper.
__global__ void k_layer_flags(const int* count, const int* pw, const unsigned char* upper, long cells, int* flags) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int f = 0;
  if (k < cells)
    for (int i = 0; i < count[k]; ++i) f |= upper[pw[k * MAX_PASSES + i]] ? 2 : 1;
  f = __reduce_or_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

struct FillArgs {
  const double *route, *cos_h, *sin_h, *grade;
  const int *nearest, *count, *pw;
  const unsigned char* upper;
  double half_width, bank, x0, y0, cell;
  int nx, layers, layer_lo, layer_hi;
  long cells;
  double *clearance, *height;  // [layers][cells]
  int* waypoint;               // [layers][cells]
};

// racer/track.py:94-104: off the road clearance -10, height 0 and the nearest
// waypoint; on it, each pass's clearance, height and waypoint (a later pass
// of the same layer overwrites an earlier one).
__global__ void k_fill(FillArgs a) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= a.cells) return;
  for (int l = 0; l < a.layers; ++l) {
    a.clearance[l * a.cells + k] = -10.0;
    a.height[l * a.cells + k] = 0.0;
    a.waypoint[l * a.cells + k] = a.nearest[k];
  }
  const double x = cell_x(a.x0, a.cell, (int)(k % a.nx)), y = cell_x(a.y0, a.cell, (int)(k / a.nx));
  for (int i = 0; i < a.count[k]; ++i) {
    const int w = a.pw[k * MAX_PASSES + i];
    const int l = a.upper[w] ? a.layer_hi : a.layer_lo;
    const double dx = x - a.route[3 * w], dy = y - a.route[3 * w + 1];
    const double c = a.cos_h[w], s = a.sin_h[w];
    const double along = dx * c + dy * s, left = -dx * s + dy * c;
    a.clearance[l * a.cells + k] = a.half_width - fabs(left);
    a.height[l * a.cells + k] = a.route[3 * w + 2] + a.grade[w] * along - a.bank * left;
    a.waypoint[l * a.cells + k] = w;
  }
}

// racer/track.py:111-117: each ramp's sloped top added to every layer's height.
__global__ void k_ramps(const RampRow* ramps, int n, double x0, double y0, double cell, int nx, long cells, int layers,
                        double* height) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= cells) return;
  const double x = cell_x(x0, cell, (int)(k % nx)), y = cell_x(y0, cell, (int)(k / nx));
  for (int r = 0; r < n; ++r) {
    const RampRow p = ramps[r];
    const double rx = x - p.cx, ry = y - p.cy;
    const double v = -rx * p.s + ry * p.c;
    double add = 0.0;  // outside the box the reference adds +0.0 too
    if (fabs(v) < p.width / 2) {
      const double u = rx * p.c + ry * p.s + p.length / 2;
      const double q = fmin(u, p.length - u) / p.rise;
      add = p.height * fmin(fmax(q, 0.0), 1.0);
    }
    for (int l = 0; l < layers; ++l) height[l * cells + k] += add;
  }
}

__global__ void k_mask_road(const double* clearance, long cells, unsigned char* feature) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < cells) feature[k] = clearance[k] > 0.0;
}

__global__ void k_mask_image(const unsigned char* free_, long cells, unsigned char* wall, unsigned char* open) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < cells) wall[k] = free_[k] == 0, open[k] = free_[k] != 0;
}

// Per column, the nearest feature row (ties to the lower row), -1 if none: one
// warp per column, the last feature at or above each row as a running
// maximum over chunks of 32 rows, then the first at or below as a running
// minimum from the bottom.
constexpr int FT_WARPS = 8;
__global__ void __launch_bounds__(FT_WARPS * 32) k_ft_columns(const unsigned char* feature, int ny, int nx, int* fy) {
  const int x = blockIdx.x * FT_WARPS + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (x >= nx) return;  // warp-uniform
  int carry = -1;
  for (int y0 = 0; y0 < ny; y0 += 32) {
    const int y = y0 + lane;
    int p = (y < ny && feature[(long)y * nx + x]) ? y : -1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int q = __shfl_up_sync(0xffffffffu, p, o);
      if (lane >= o) p = max(p, q);
    }
    p = max(p, carry);
    if (y < ny) fy[(long)y * nx + x] = p;
    carry = __shfl_sync(0xffffffffu, p, 31);
  }
  int below = INT_MAX;
  for (int y0 = ((ny - 1) / 32) * 32; y0 >= 0; y0 -= 32) {
    const int y = y0 + lane;
    int q = (y < ny && feature[(long)y * nx + x]) ? y : INT_MAX;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int r = __shfl_down_sync(0xffffffffu, q, o);
      if (lane + o < 32) q = min(q, r);
    }
    q = min(q, below);
    if (y < ny && q != INT_MAX) {
      const int p = fy[(long)y * nx + x];
      if (p < 0 || q - y < y - p) fy[(long)y * nx + x] = q;
    }
    below = __shfl_sync(0xffffffffu, q, 0);
  }
}

__device__ void ft_row(const int* row, int y, int nx, int* gs, int* out) {
  int l = -1;
  for (int x = 0; x < nx; ++x) {
    const int fx = row[x];
    if (fx < 0) continue;
    const long long wR = (long long)(fx - y) * (fx - y);
    while (l >= 1) {
      const int v = gs[l], u = gs[l - 1];
      const long long a = v - u, b = x - v, c = a + b;
      const long long vR = (long long)(row[v] - y) * (row[v] - y), uR = (long long)(row[u] - y) * (row[u] - y);
      if (c * vR - b * uR - a * wR - a * b * c <= 0) break;
      --l;
    }
    gs[++l] = x;
  }
  if (l < 0) {
    for (int x = 0; x < nx; ++x) out[x] = -1;
    return;
  }
  const int maxl = l;
  l = 0;
  for (int x = 0; x < nx; ++x) {
    int gl = gs[l];
    long long d1 = (long long)(gl - x) * (gl - x) + (long long)(row[gl] - y) * (row[gl] - y);
    while (l < maxl) {
      const int gn = gs[l + 1];
      const long long d2 = (long long)(gn - x) * (gn - x) + (long long)(row[gn] - y) * (row[gn] - y);
      if (d1 <= d2) break;
      d1 = d2, ++l, gl = gn;
    }
    out[x] = row[gl] * nx + gl;
  }
}

// Per row, the lower envelope of the columns' candidates and, for every cell,
// the flat index of its nearest feature (-1 when the grid has none). The
// envelope is sequential: one thread walks the row, in shared memory when
// SHARED (a warp per row stages the row, its stack and its output there),
// else in global memory (`g` holds the stacks).
template <bool SHARED>
__global__ void k_ft_rows(const int* fy, int ny, int nx, int* g, int* src) {
  extern __shared__ int ft_smem[];
  const int y = SHARED ? blockIdx.x : blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  const int* row = fy + (long)y * nx;
  int* gs = g + (long)y * nx;
  int* out = src + (long)y * nx;
  if (SHARED) {
    for (int x = threadIdx.x; x < nx; x += 32) ft_smem[x] = row[x];
    __syncwarp();
    row = ft_smem, gs = ft_smem + nx, out = ft_smem + 2 * nx;
    if (threadIdx.x == 0) ft_row(row, y, nx, gs, out);
    __syncwarp();
    for (int x = threadIdx.x; x < nx; x += 32) src[(long)y * nx + x] = out[x];
    return;
  }
  ft_row(row, y, nx, gs, out);
}

__global__ void k_gather(const double* height, const int* src, long cells, double* filled) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < cells) filled[k] = height[src[k]];
}

__device__ __forceinline__ int reflect(int i, int n) {
  int m = i % (2 * n);
  if (m < 0) m += 2 * n;
  return m >= n ? 2 * n - 1 - m : m;
}

__global__ void k_blur_rows(const double* in, int ny, int nx, Blur b, double* out) {  // along axis 0
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= (long)nx * ny) return;
  const int x = (int)(k % nx), y = (int)(k / nx);
  double s = in[k] * b.w[6];
#pragma unroll
  for (int j = 6; j >= 1; --j)
    s += (in[(long)reflect(y - j, ny) * nx + x] + in[(long)reflect(y + j, ny) * nx + x]) * b.w[6 - j];
  out[k] = s;
}

__global__ void k_blur_cols(const double* in, int ny, int nx, Blur b, float* out) {  // along axis 1, to float32
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= (long)nx * ny) return;
  const int x = (int)(k % nx);
  const double* r = in + (k - x);
  double s = r[x] * b.w[6];
#pragma unroll
  for (int j = 6; j >= 1; --j) s += (r[reflect(x - j, nx)] + r[reflect(x + j, nx)]) * b.w[6 - j];
  out[k] = (float)s;
}

__global__ void k_write_layer(const double* clearance, const int* waypoint, long cells, float* out) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= cells) return;
  out[k] = (float)clearance[k];
  out[2 * cells + k] = (float)waypoint[k];
}

// racer/track.py:57: (distance to the nearest wall - distance to the nearest
// free cell - 0.5) * cell, distances from the feature transforms.
__global__ void k_image_clear(const unsigned char* free_, const int* to_wall, const int* to_open, int nx, long cells,
                              double cell, double* clearance) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= cells) return;
  const int f = free_[k] ? to_wall[k] : to_open[k];
  const double dy = (double)(f / nx) - (double)(k / nx), dx = (double)(f % nx) - (double)(k % nx);
  const double d = sqrt(dy * dy + dx * dx);
  const double a = free_[k] ? d : 0.0, b = free_[k] ? 0.0 : d;
  clearance[k] = (a - b - 0.5) * cell;
}

Blur blur_weights() {  // sigma 1.5, radius 6
  const double sigma = 1.5;
  double phi[13];
  for (int i = 0; i < 13; ++i) {
    const double x = i - 6;
    phi[i] = std::exp(-0.5 / (sigma * sigma) * (x * x));
  }
  // the sum in pairwise order: eight leading terms as a tree, then the rest in turn
  double sum = ((phi[0] + phi[1]) + (phi[2] + phi[3])) + ((phi[4] + phi[5]) + (phi[6] + phi[7]));
  for (int i = 8; i < 13; ++i) sum += phi[i];
  Blur b;
  for (int i = 0; i < 13; ++i) b.w[i] = phi[i] / sum;
  return b;
}

// Device buffers of one compilation, freed on every exit path.
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t get(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T) + 16);
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

inline unsigned blocks(long n, int t) { return (unsigned)((n + t - 1) / t); }

// The feature transform of `feature` into `src` (flat index of each cell's
// nearest feature); fy and g are [cells] scratch.
cudaError_t feature_transform(const unsigned char* feature, int ny, int nx, int* fy, int* g, int* src, cudaStream_t st) {
  k_ft_columns<<<blocks(nx, FT_WARPS), FT_WARPS * 32, 0, st>>>(feature, ny, nx, fy);
  const size_t smem = 3 * sizeof(int) * (size_t)nx;
  if (smem <= 48 * 1024 ||
      (smem <= 200 * 1024 &&
       cudaFuncSetAttribute(k_ft_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess)) {
    k_ft_rows<true><<<ny, 32, smem, st>>>(fy, ny, nx, g, src);
  } else {
    cudaGetLastError();
    k_ft_rows<false><<<blocks(ny, 64), 64, 0, st>>>(fy, ny, nx, g, src);
  }
  return cudaGetLastError();
}

#define TRACK_LAUNCH()                                                                            \
  do {                                                                                            \
    cudaError_t e_ = cudaGetLastError();                                                          \
    if (e_ != cudaSuccess) {                                                                      \
      racer_host::set_error(std::string("track kernel launch: ") + cudaGetErrorString(e_));       \
      return 2;                                                                                   \
    }                                                                                             \
  } while (0)

// racer/track.py:108-125 from the device grids: ramps, off-road fill, blur,
// float32 grids [layers][3][cells] into `grids` (device).
int pack(Scratch& s, int layers, double* clearance, double* height, const int* waypoint, const RampRow* ramps_dev,
         int n_ramps, double x0, double y0, double cell, int nx, int ny, float* grids, cudaStream_t st) {
  const long cells = (long)nx * ny;
  const int T = 256;
  if (n_ramps) {
    k_ramps<<<blocks(cells, T), T, 0, st>>>(ramps_dev, n_ramps, x0, y0, cell, nx, cells, layers, height);
    TRACK_LAUNCH();
  }
  unsigned char* feature;
  int *fy, *g, *src;
  double *filled, *tmp;
  RACER_TRY(s.get(&feature, cells));
  RACER_TRY(s.get(&fy, cells));
  RACER_TRY(s.get(&g, cells));
  RACER_TRY(s.get(&src, cells));
  RACER_TRY(s.get(&filled, cells));
  RACER_TRY(s.get(&tmp, cells));
  const Blur b = blur_weights();
  for (int l = 0; l < layers; ++l) {
    k_mask_road<<<blocks(cells, T), T, 0, st>>>(clearance + l * cells, cells, feature);
    RACER_TRY(feature_transform(feature, ny, nx, fy, g, src, st));
    TRACK_LAUNCH();
    int first = 0;
    RACER_TRY(cudaMemcpyAsync(&first, src, sizeof(int), cudaMemcpyDeviceToHost, st));
    RACER_TRY(cudaStreamSynchronize(st));
    if (first < 0) {
      racer_host::set_error("track: a layer has no road cell (clearance > 0)");
      return 3;
    }
    float* out = grids + (long)l * 3 * cells;
    k_gather<<<blocks(cells, T), T, 0, st>>>(height + l * cells, src, cells, filled);
    k_blur_rows<<<blocks(cells, T), T, 0, st>>>(filled, ny, nx, b, tmp);
    k_blur_cols<<<blocks(cells, T), T, 0, st>>>(tmp, ny, nx, b, out + cells);
    k_write_layer<<<blocks(cells, T), T, 0, st>>>(clearance + l * cells, waypoint + l * cells, cells, out);
    TRACK_LAUNCH();
  }
  return 0;
}

struct Stream {
  cudaStream_t s = nullptr;
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
};

bool grid_ok(int nx, int ny) { return nx >= 2 && ny >= 2 && (long)nx * ny <= (1L << 30) / 8; }

}  // namespace

extern "C" {

int racer_track_ribbon(const double* route, const double* cos_h, const double* sin_h, const double* grade, int W,
                       double half_width, double bank, double x0, double y0, double cell, int nx, int ny,
                       const double* ramps, int n_ramps, float* grids, int64_t grids_len, int* layers_out) {
  if (!route || !cos_h || !sin_h || !grade || !grids || !layers_out || W < 2 || !grid_ok(nx, ny) || !(cell > 0) ||
      n_ramps < 0 || (n_ramps && !ramps)) {
    racer_host::set_error("racer_track_ribbon: invalid arguments");
    return 1;
  }
  const long cells = (long)nx * ny;
  if (grids_len < 6 * cells) {
    racer_host::set_error("racer_track_ribbon: grids needs 6 * nx * ny floats");
    return 1;
  }
  Stream st;
  RACER_TRY(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
  Scratch s;
  double *d_route, *d_cos, *d_sin, *d_grade;
  int *nearest, *count, *pw, *flags;
  unsigned char* upper;
  RACER_TRY(s.get(&d_route, 3 * (size_t)W));
  RACER_TRY(s.get(&d_cos, W));
  RACER_TRY(s.get(&d_sin, W));
  RACER_TRY(s.get(&d_grade, W));
  RACER_TRY(s.get(&nearest, cells));
  RACER_TRY(s.get(&count, cells));
  RACER_TRY(s.get(&pw, cells * MAX_PASSES));
  RACER_TRY(s.get(&flags, 2));
  RACER_TRY(s.get(&upper, W));
  RACER_TRY(cudaMemcpyAsync(d_route, route, 3 * sizeof(double) * W, cudaMemcpyHostToDevice, st.s));
  RACER_TRY(cudaMemcpyAsync(d_cos, cos_h, sizeof(double) * W, cudaMemcpyHostToDevice, st.s));
  RACER_TRY(cudaMemcpyAsync(d_sin, sin_h, sizeof(double) * W, cudaMemcpyHostToDevice, st.s));
  RACER_TRY(cudaMemcpyAsync(d_grade, grade, sizeof(double) * W, cudaMemcpyHostToDevice, st.s));
  RACER_TRY(cudaMemsetAsync(flags, 0, 2 * sizeof(int), st.s));
  RACER_TRY(cudaMemsetAsync(upper, 0, W, st.s));

  const double r = half_width + 0.5;
  CellArgs ca{d_route, W, x0, y0, cell, nx, ny, r * r, nearest, count, pw, upper, flags + 1};
  k_cells<<<dim3(blocks(nx, TILE), blocks(ny, TILE)), TILE * TILE, 0, st.s>>>(ca);
  TRACK_LAUNCH();

  // racer/track.py:88-93: the upper layer grows along the route while it stays raised
  std::vector<unsigned char> up(W), grown(W);
  int err = 0;
  RACER_TRY(cudaMemcpyAsync(up.data(), upper, W, cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaMemcpyAsync(&err, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaStreamSynchronize(st.s));
  if (err) {
    racer_host::set_error("racer_track_ribbon: a cell lies under more than 8 passes of the route");
    return 4;
  }
  double zmin = route[2];
  for (int w = 1; w < W; ++w) zmin = std::fmin(zmin, route[3 * w + 2]);
  for (;;) {
    bool same = true;
    for (int w = 0; w < W; ++w) {
      const unsigned char high = route[3 * w + 2] > zmin + 0.1;
      grown[w] = up[w] | ((up[(w + W - 1) % W] | up[(w + 1) % W]) & high);
      same = same && grown[w] == up[w];
    }
    if (same) break;
    up.swap(grown);
  }
  RACER_TRY(cudaMemcpyAsync(upper, up.data(), W, cudaMemcpyHostToDevice, st.s));
  k_layer_flags<<<blocks(cells, 256), 256, 0, st.s>>>(count, pw, upper, cells, flags);
  TRACK_LAUNCH();
  int f = 0;
  RACER_TRY(cudaMemcpyAsync(&f, flags, sizeof(int), cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaStreamSynchronize(st.s));
  const int layers = (f & 1) + ((f >> 1) & 1);
  if (layers == 0) {
    racer_host::set_error("racer_track_ribbon: no cell lies on the road");
    return 3;
  }
  double *clearance, *height;
  int* waypoint;
  float* d_grids;
  RampRow* d_ramps = nullptr;
  RACER_TRY(s.get(&clearance, layers * cells));
  RACER_TRY(s.get(&height, layers * cells));
  RACER_TRY(s.get(&waypoint, layers * cells));
  RACER_TRY(s.get(&d_grids, 3 * layers * cells));
  if (n_ramps) {
    RACER_TRY(s.get(&d_ramps, n_ramps));
    RACER_TRY(cudaMemcpyAsync(d_ramps, ramps, sizeof(RampRow) * n_ramps, cudaMemcpyHostToDevice, st.s));
  }
  FillArgs fa{d_route, d_cos, d_sin, d_grade, nearest, count, pw, upper, half_width, bank, x0, y0, cell,
              nx, layers, 0, (f & 1) ? 1 : 0, cells, clearance, height, waypoint};
  k_fill<<<blocks(cells, 256), 256, 0, st.s>>>(fa);
  TRACK_LAUNCH();
  int rc = pack(s, layers, clearance, height, waypoint, d_ramps, n_ramps, x0, y0, cell, nx, ny, d_grids, st.s);
  if (rc) return rc;
  RACER_TRY(cudaMemcpyAsync(grids, d_grids, sizeof(float) * 3 * layers * cells, cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaStreamSynchronize(st.s));
  *layers_out = layers;
  return 0;
}

int racer_track_image(const uint8_t* free_, const double* route, int W, double x0, double y0, double cell, int nx,
                      int ny, const double* ramps, int n_ramps, float* grids, int64_t grids_len) {
  if (!free_ || !route || !grids || W < 1 || !grid_ok(nx, ny) || !(cell > 0) || n_ramps < 0 ||
      (n_ramps && !ramps)) {
    racer_host::set_error("racer_track_image: invalid arguments");
    return 1;
  }
  const long cells = (long)nx * ny;
  if (grids_len < 3 * cells) {
    racer_host::set_error("racer_track_image: grids needs 3 * nx * ny floats");
    return 1;
  }
  Stream st;
  RACER_TRY(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
  Scratch s;
  double *d_route, *clearance, *height;
  unsigned char *d_free, *wall, *open;
  int *nearest, *to_wall, *to_open, *fy, *g, *flags;
  float* d_grids;
  RampRow* d_ramps = nullptr;
  RACER_TRY(s.get(&d_route, 3 * (size_t)W));
  RACER_TRY(s.get(&d_free, cells));
  RACER_TRY(s.get(&wall, cells));
  RACER_TRY(s.get(&open, cells));
  RACER_TRY(s.get(&nearest, cells));
  RACER_TRY(s.get(&to_wall, cells));
  RACER_TRY(s.get(&to_open, cells));
  RACER_TRY(s.get(&fy, cells));
  RACER_TRY(s.get(&g, cells));
  RACER_TRY(s.get(&flags, 2));
  RACER_TRY(s.get(&clearance, cells));
  RACER_TRY(s.get(&height, cells));
  RACER_TRY(s.get(&d_grids, 3 * cells));
  RACER_TRY(cudaMemcpyAsync(d_route, route, 3 * sizeof(double) * W, cudaMemcpyHostToDevice, st.s));
  RACER_TRY(cudaMemcpyAsync(d_free, free_, cells, cudaMemcpyHostToDevice, st.s));
  RACER_TRY(cudaMemsetAsync(flags, 0, 2 * sizeof(int), st.s));
  RACER_TRY(cudaMemsetAsync(height, 0, sizeof(double) * cells, st.s));
  if (n_ramps) {
    RACER_TRY(s.get(&d_ramps, n_ramps));
    RACER_TRY(cudaMemcpyAsync(d_ramps, ramps, sizeof(RampRow) * n_ramps, cudaMemcpyHostToDevice, st.s));
  }
  CellArgs ca{d_route, W, x0, y0, cell, nx, ny, -1.0, nearest, nullptr, nullptr, nullptr, flags + 1};
  k_cells<<<dim3(blocks(nx, TILE), blocks(ny, TILE)), TILE * TILE, 0, st.s>>>(ca);
  k_mask_image<<<blocks(cells, 256), 256, 0, st.s>>>(d_free, cells, wall, open);
  TRACK_LAUNCH();
  RACER_TRY(feature_transform(wall, ny, nx, fy, g, to_wall, st.s));
  RACER_TRY(feature_transform(open, ny, nx, fy, g, to_open, st.s));
  int first[2] = {0, 0};
  RACER_TRY(cudaMemcpyAsync(&first[0], to_wall, sizeof(int), cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaMemcpyAsync(&first[1], to_open, sizeof(int), cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaStreamSynchronize(st.s));
  if (first[0] < 0 || first[1] < 0) {
    racer_host::set_error("racer_track_image: the image needs both free and occupied cells");
    return 3;
  }
  k_image_clear<<<blocks(cells, 256), 256, 0, st.s>>>(d_free, to_wall, to_open, nx, cells, cell, clearance);
  TRACK_LAUNCH();
  int rc = pack(s, 1, clearance, height, nearest, d_ramps, n_ramps, x0, y0, cell, nx, ny, d_grids, st.s);
  if (rc) return rc;
  RACER_TRY(cudaMemcpyAsync(grids, d_grids, sizeof(float) * 3 * cells, cudaMemcpyDeviceToHost, st.s));
  RACER_TRY(cudaStreamSynchronize(st.s));
  return 0;
}

}  // extern "C"
