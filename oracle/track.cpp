// CPU oracle of the track compiler (TEST INFRASTRUCTURE ONLY): a C++
// restatement of the per-cell work of racer/track.py (cells in parallel under
// OpenMP, each as the reference's loop computes it), checked against arrays
// that the reference's own compiler produced.
//
//   orc_track_ribbon   racer/track.py:61-105 (ribbon) + :108-125 (pack)
//   orc_track_image    racer/track.py:54-58 (occupancy image) + :108-125
//
// The per-waypoint inputs (resampled route, cos/sin of the headings, grade)
// and the header are computed by the caller in numpy exactly as the reference
// does, so this file holds only the per-cell arithmetic. The nearest-waypoint
// searches that the reference runs through scipy's KDTree are brute force
// here; the feature transform and the Gaussian blur that it runs through
// scipy.ndimage are restated: the feature transform is the separable exact
// Euclidean method of Maurer, Qi and Raghavan (2003), axis 0 first, ties to
// the lower index; the blur is a 13-tap correlation (sigma 1.5, radius 6,
// weights exp(-x^2 / 2 sigma^2) / sum), reflected at the edges, axis 0 then
// axis 1, each output summed as centre tap, then symmetric pairs from the
// outermost inward. All arithmetic is binary64 without contraction.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int MAX_PASSES = 8;

struct Ramp {
  double cx, cy, c, s, length, width, height, rise;
};

// Index of the waypoint nearest (x, y), the lowest index among equals
// (racer/track.py:89 and :56, KDTree.query).
int nearest_waypoint(const double* route, int W, double x, double y) {
  int best = 0;
  double bd = INFINITY;
  for (int w = 0; w < W; ++w) {
    double dx = route[3 * w] - x, dy = route[3 * w + 1] - y;
    double d2 = dx * dx + dy * dy;
    if (d2 < bd) bd = d2, best = w;
  }
  return best;
}

// The passes of the route over one cell and the nearest waypoint of each,
// reduced to the layers the cell belongs to (racer/track.py:73-86). Returns
// the count written to `out` (0 off the road), -1 on too many passes.
int cell_nearest(const double* route, int W, double x, double y, double r2, int* out) {
  int pbest[MAX_PASSES];
  double pd[MAX_PASSES];
  int np = 0, first = -1, last = -10;
  for (int w = 0; w < W; ++w) {
    double dx = route[3 * w] - x, dy = route[3 * w + 1] - y;
    double d2 = dx * dx + dy * dy;
    if (!(d2 <= r2)) continue;
    double d = std::sqrt(d2);
    if (np == 0 || w - last > 2) {  // a gap of more than 2 starts a new pass
      if (np == MAX_PASSES) return -1;
      pbest[np] = w, pd[np] = d, ++np;
    } else if (d < pd[np - 1]) {
      pbest[np - 1] = w, pd[np - 1] = d;
    }
    if (first < 0) first = w;
    last = w;
  }
  if (np == 0) return 0;
  if (np > 1 && first == 0 && last == W - 1) {  // the pass through the seam: its end, then its start
    int bw = pbest[np - 1];
    double bd = pd[np - 1];
    if (pd[0] < bd) bw = pbest[0], bd = pd[0];
    pbest[0] = bw, pd[0] = bd, --np;
  }
  for (int i = 1; i < np; ++i) {  // stable sort by height
    int w = pbest[i];
    double d = pd[i];
    int j = i;
    while (j > 0 && route[3 * pbest[j - 1] + 2] > route[3 * w + 2]) pbest[j] = pbest[j - 1], pd[j] = pd[j - 1], --j;
    pbest[j] = w, pd[j] = d;
  }
  if (route[3 * pbest[np - 1] + 2] - route[3 * pbest[0] + 2] < 0.3) {  // one level: the nearest pass
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

// Nearest feature of every cell of an ny x nx grid (feature[k] != 0), as a
// flat index, or -1 when the grid has no feature.
void feature_transform(const uint8_t* feature, int ny, int nx, std::vector<int>& nearest) {
  std::vector<int> fy((size_t)ny * nx, -1);
  for (int x = 0; x < nx; ++x) {  // axis 0: nearest feature row in the column, ties to the lower row
    int prev = -1;
    for (int y = 0; y < ny; ++y) {
      if (feature[(size_t)y * nx + x]) prev = y;
      fy[(size_t)y * nx + x] = prev;
    }
    int next = -1;
    for (int y = ny - 1; y >= 0; --y) {
      if (feature[(size_t)y * nx + x]) next = y;
      int p = fy[(size_t)y * nx + x];
      if (next >= 0 && (p < 0 || next - y < y - p)) fy[(size_t)y * nx + x] = next;
    }
  }
  nearest.assign((size_t)ny * nx, -1);
  std::vector<int> g(nx);
  for (int y = 0; y < ny; ++y) {  // axis 1: lower envelope of the columns' candidates
    const int* row = &fy[(size_t)y * nx];
    int l = -1;
    for (int x = 0; x < nx; ++x) {
      if (row[x] < 0) continue;
      long long wR = (long long)(row[x] - y) * (row[x] - y);
      while (l >= 1) {
        int v = g[l], u = g[l - 1];
        long long a = v - u, b = x - v, c = a + b;
        long long vR = (long long)(row[v] - y) * (row[v] - y), uR = (long long)(row[u] - y) * (row[u] - y);
        if (c * vR - b * uR - a * wR - a * b * c <= 0) break;
        --l;
      }
      g[++l] = x;
    }
    if (l < 0) continue;
    int maxl = l;
    l = 0;
    for (int x = 0; x < nx; ++x) {
      long long d1 = (long long)(g[l] - x) * (g[l] - x) + (long long)(row[g[l]] - y) * (row[g[l]] - y);
      while (l < maxl) {
        long long d2 = (long long)(g[l + 1] - x) * (g[l + 1] - x) + (long long)(row[g[l + 1]] - y) * (row[g[l + 1]] - y);
        if (d1 <= d2) break;
        d1 = d2, ++l;
      }
      nearest[(size_t)y * nx + x] = row[g[l]] * nx + g[l];
    }
  }
}

void blur_weights(double* w) {  // 13 taps of sigma 1.5
  const double sigma = 1.5;
  double phi[13];
  for (int i = 0; i < 13; ++i) {
    double x = i - 6;
    phi[i] = std::exp(-0.5 / (sigma * sigma) * (x * x));
  }
  // the sum in pairwise order: eight leading terms as a tree, then the rest in turn
  double sum = ((phi[0] + phi[1]) + (phi[2] + phi[3])) + ((phi[4] + phi[5]) + (phi[6] + phi[7]));
  for (int i = 8; i < 13; ++i) sum += phi[i];
  for (int i = 0; i < 13; ++i) w[i] = phi[i] / sum;
}

inline int reflect(int i, int n) {
  int m = i % (2 * n);
  if (m < 0) m += 2 * n;
  return m >= n ? 2 * n - 1 - m : m;
}

void blur(std::vector<double>& a, int ny, int nx) {
  double w[13];
  blur_weights(w);
  std::vector<double> t(a.size());
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      double s = a[(size_t)y * nx + x] * w[6];
      for (int j = 6; j >= 1; --j)
        s += (a[(size_t)reflect(y - j, ny) * nx + x] + a[(size_t)reflect(y + j, ny) * nx + x]) * w[6 - j];
      t[(size_t)y * nx + x] = s;
    }
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const double* r = &t[(size_t)y * nx];
      double s = r[x] * w[6];
      for (int j = 6; j >= 1; --j) s += (r[reflect(x - j, nx)] + r[reflect(x + j, nx)]) * w[6 - j];
      a[(size_t)y * nx + x] = s;
    }
}

// racer/track.py:108-125 without the header and route: ramps, off-road fill
// from the nearest road cell, blur, float32 grids [layers][3][ny * nx].
int pack(int layers, std::vector<double>& clearance, std::vector<double>& height, const std::vector<int>& waypoint,
         double x0, double y0, double cell, int nx, int ny, const Ramp* ramps, int n_ramps, float* grids) {
  const size_t cells = (size_t)nx * ny;
  for (int r = 0; r < n_ramps; ++r) {
    const Ramp& p = ramps[r];
    for (size_t k = 0; k < cells; ++k) {
      double rx = (x0 + cell * (double)(k % nx)) - p.cx, ry = (y0 + cell * (double)(k / nx)) - p.cy;
      double u = rx * p.c + ry * p.s + p.length / 2;
      double v = -rx * p.s + ry * p.c;
      double q = std::fmin(u, p.length - u) / p.rise;
      double top = p.height * std::fmin(std::fmax(q, 0.0), 1.0);
      double add = std::fabs(v) < p.width / 2 ? top : 0.0;
      for (int l = 0; l < layers; ++l) height[l * cells + k] += add;
    }
  }
  std::vector<uint8_t> road(cells);
  std::vector<int> src;
  std::vector<double> filled(cells);
  for (int l = 0; l < layers; ++l) {
    for (size_t k = 0; k < cells; ++k) road[k] = clearance[l * cells + k] > 0;
    feature_transform(road.data(), ny, nx, src);
    if (src[0] < 0) return 3;  // a layer without road
    for (size_t k = 0; k < cells; ++k) filled[k] = height[l * cells + src[k]];
    blur(filled, ny, nx);
    float* out = grids + (size_t)l * 3 * cells;
    for (size_t k = 0; k < cells; ++k) {
      out[k] = (float)clearance[l * cells + k];
      out[cells + k] = (float)filled[k];
      out[2 * cells + k] = (float)waypoint[l * cells + k];
    }
  }
  return 0;
}

}  // namespace

extern "C" {

// Grids of a ribbon track (racer/track.py:61-105, then pack :108-125).
// route [W][3] resampled, cos_h/sin_h of the headings, grade [W];
// ramps [n_ramps][8] = (cx, cy, cos, sin, length, width, height, rise).
// Writes [layers][3][ny * nx] floats (grids_len >= 6 * nx * ny) and *layers.
int orc_track_ribbon(const double* route, const double* cos_h, const double* sin_h, const double* grade, int W,
                     double half_width, double bank, double x0, double y0, double cell, int nx, int ny,
                     const double* ramps, int n_ramps, float* grids, long grids_len, int* layers_out) {
  const size_t cells = (size_t)nx * ny;
  if (W < 2 || nx < 2 || ny < 2 || grids_len < (long)(6 * cells)) return 1;
  const double r = half_width + 0.5, r2 = r * r;
  std::vector<int> nearest(cells), count(cells), kept(cells * MAX_PASSES);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : bad)
  for (long k = 0; k < (long)cells; ++k) {
    double x = x0 + cell * (double)(k % nx), y = y0 + cell * (double)(k / nx);
    nearest[k] = nearest_waypoint(route, W, x, y);
    count[k] = cell_nearest(route, W, x, y, r2, &kept[k * MAX_PASSES]);
    bad |= count[k] < 0;
  }
  if (bad) return 2;
  std::vector<int> pair_cell, pair_w;  // in the reference's order: by cell, then by height
  std::vector<uint8_t> upper(W, 0);
  for (size_t k = 0; k < cells; ++k)
    for (int i = 0; i < count[k]; ++i) {
      int w = kept[k * MAX_PASSES + i];
      if (i > 0) upper[w] = 1;
      pair_cell.push_back((int)k), pair_w.push_back(w);
    }
  double zmin = route[2];
  for (int w = 1; w < W; ++w) zmin = std::fmin(zmin, route[3 * w + 2]);
  std::vector<uint8_t> grown(W);
  for (;;) {  // racer/track.py:88-93
    bool same = true;
    for (int w = 0; w < W; ++w) {
      bool high = route[3 * w + 2] > zmin + 0.1;
      grown[w] = upper[w] | ((upper[(w + W - 1) % W] | upper[(w + 1) % W]) & (uint8_t)high);
      same = same && grown[w] == upper[w];
    }
    if (same) break;
    upper = grown;
  }
  bool any_low = false, any_high = false;
  for (int w : pair_w) (upper[w] ? any_high : any_low) = true;
  const int layers = any_low + any_high;
  if (layers == 0) return 3;
  const int layer_of[2] = {0, any_low ? 1 : 0};
  std::vector<double> clearance(layers * cells, -10.0), height(layers * cells, 0.0);
  std::vector<int> waypoint(layers * cells);
  for (int l = 0; l < layers; ++l) std::memcpy(&waypoint[l * cells], nearest.data(), cells * sizeof(int));
  for (size_t i = 0; i < pair_w.size(); ++i) {
    int k = pair_cell[i], w = pair_w[i], l = layer_of[upper[w]];
    double dx = (x0 + cell * (double)(k % nx)) - route[3 * w], dy = (y0 + cell * (double)(k / nx)) - route[3 * w + 1];
    double along = dx * cos_h[w] + dy * sin_h[w], left = -dx * sin_h[w] + dy * cos_h[w];
    clearance[l * cells + k] = half_width - std::fabs(left);
    height[l * cells + k] = route[3 * w + 2] + grade[w] * along - bank * left;
    waypoint[l * cells + k] = w;
  }
  *layers_out = layers;
  return pack(layers, clearance, height, waypoint, x0, y0, cell, nx, ny, (const Ramp*)ramps, n_ramps, grids);
}

// Grids of an occupancy-image track (racer/track.py:54-58, then pack):
// free [ny * nx] (rows south to north), route [W][3] resampled.
int orc_track_image(const uint8_t* free_, const double* route, int W, double x0, double y0, double cell, int nx, int ny,
                    const double* ramps, int n_ramps, float* grids, long grids_len) {
  const size_t cells = (size_t)nx * ny;
  if (W < 1 || nx < 2 || ny < 2 || grids_len < (long)(3 * cells)) return 1;
  std::vector<uint8_t> wall(cells), open(cells);
  for (size_t k = 0; k < cells; ++k) open[k] = free_[k] != 0, wall[k] = free_[k] == 0;
  std::vector<int> to_wall, to_open;
  feature_transform(wall.data(), ny, nx, to_wall);
  feature_transform(open.data(), ny, nx, to_open);
  if (to_wall[0] < 0 || to_open[0] < 0) return 3;
  std::vector<double> clearance(cells), height(cells, 0.0);
  std::vector<int> waypoint(cells);
  auto dist = [nx](size_t k, int f) {
    double dy = (double)(f / nx) - (double)(k / nx), dx = (double)(f % nx) - (double)(k % nx);
    return std::sqrt(dy * dy + dx * dx);
  };
#pragma omp parallel for schedule(dynamic, 4096)
  for (long k = 0; k < (long)cells; ++k) {
    double a = open[k] ? dist(k, to_wall[k]) : 0.0, b = open[k] ? 0.0 : dist(k, to_open[k]);
    clearance[k] = (a - b - 0.5) * cell;
    waypoint[k] = nearest_waypoint(route, W, x0 + cell * (double)(k % nx), y0 + cell * (double)(k / nx));
  }
  return pack(1, clearance, height, waypoint, x0, y0, cell, nx, ny, (const Ramp*)ramps, n_ramps, grids);
}

}  // extern "C"
