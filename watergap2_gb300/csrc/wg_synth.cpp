// wg_synth.cpp -- host-side generator helpers for large synthetic regions
// (libwg_synth.so): priority-flood pit filling and D8 steepest descent.
//
// Same algorithm, tie-breaking and arithmetic as flood_and_d8() in
// watergap2_gb300/synthetic.py (which it replaces for grids too large for a
// Python loop): cells enter a min-heap ordered by (filled elevation, row,
// column); a neighbour reached from a cell gets max(own elevation, that
// elevation + 1e-6); land never reached from a seed (an island) gets its lowest
// cell as an extra outlet; then each non-seed land cell drains to the
// neighbour with the steepest drop (diagonals divided by sqrt 2, first maximum
// in row-major neighbour order).  LDD codes follow the reference's keypad
// convention (source/rout_prepare.cpp:619-670): 5 at outlets.
#include <cmath>
#include <cstdint>
#include <queue>
#include <vector>

namespace {

struct Node {
  double z;
  int r, c;
  bool operator>(const Node &o) const {
    if (z != o.z) return z > o.z;
    if (r != o.r) return r > o.r;
    return c > o.c;
  }
};

// keypad code of a step (dr, dc), rows growing southwards
int8_t code_of(int dr, int dc) {
  static const int8_t tab[3][3] = {{7, 8, 9}, {4, 5, 6}, {1, 2, 3}};
  return tab[dr + 1][dc + 1];
}

}  // namespace

extern "C" int wg_synth_flood_d8(int ny, int nx, const double *dem, const uint8_t *land, uint8_t *seeds, int wrap,
                                 int8_t *ldd_out) {
  const size_t N = (size_t)ny * nx;
  const double eps = 1e-6;
  std::vector<double> filled(N, INFINITY);
  std::vector<uint8_t> done(N, 0);
  std::priority_queue<Node, std::vector<Node>, std::greater<Node>> heap;
  for (int r = 0; r < ny; ++r)
    for (int c = 0; c < nx; ++c) {
      const size_t k = (size_t)r * nx + c;
      if (seeds[k]) {
        filled[k] = dem[k];
        done[k] = 1;
        heap.push({dem[k], r, c});
      }
    }
  size_t scan = 0;
  for (;;) {
    while (!heap.empty()) {
      const Node t = heap.top();
      heap.pop();
      for (int dr = -1; dr <= 1; ++dr)
        for (int dc = -1; dc <= 1; ++dc) {
          if (!dr && !dc) continue;
          const int rr = t.r + dr;
          int cc = t.c + dc;
          if (rr < 0 || rr >= ny) continue;
          if (cc < 0 || cc >= nx) {
            if (!wrap) continue;
            cc = (cc + nx) % nx;
          }
          const size_t k = (size_t)rr * nx + cc;
          if (!land[k] || done[k]) continue;
          done[k] = 1;
          const double zz = dem[k] > t.z + eps ? dem[k] : t.z + eps;
          filled[k] = zz;
          heap.push({zz, rr, cc});
        }
    }
    // lowest land cell not reached yet (first in row-major order on ties)
    size_t best = N;
    for (size_t k = scan; k < N; ++k)
      if (land[k] && !done[k] && (best == N || dem[k] < dem[best])) best = k;
    if (best == N) break;
    // everything before the first unreached land cell stays reached
    while (scan < N && !(land[scan] && !done[scan])) ++scan;
    seeds[best] = 1;
    done[best] = 1;
    filled[best] = dem[best];
    heap.push({dem[best], (int)(best / nx), (int)(best % nx)});
  }
  const double sq2 = std::sqrt(2.0);
  for (int r = 0; r < ny; ++r)
    for (int c = 0; c < nx; ++c) {
      const size_t k = (size_t)r * nx + c;
      ldd_out[k] = 0;
      if (!land[k]) continue;
      if (seeds[k]) {
        ldd_out[k] = 5;
        continue;
      }
      double best = 0.0;
      int8_t code = 0;
      for (int dr = -1; dr <= 1; ++dr)
        for (int dc = -1; dc <= 1; ++dc) {
          if (!dr && !dc) continue;
          const int rr = r + dr;
          int cc = c + dc;
          if (rr < 0 || rr >= ny) continue;
          if (cc < 0 || cc >= nx) {
            if (!wrap) continue;
            cc = (cc + nx) % nx;
          }
          const size_t q = (size_t)rr * nx + cc;
          if (!land[q]) continue;
          const double drop = (filled[k] - filled[q]) / ((dr && dc) ? sq2 : 1.0);
          if (drop > best) {
            best = drop;
            code = code_of(dr, dc);
          }
        }
      if (code == 0) return -1;
      ldd_out[k] = code;
    }
  return 0;
}
