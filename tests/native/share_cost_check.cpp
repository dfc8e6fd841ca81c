// Host check of fvgb::ShareCost (fv_internal.h), the step kernels' work
// distribution: for many grid shapes and warp counts, the warps' shares
// [pos(g*C/G), pos((g+1)*C/G)) tile the (window, row) positions
// 0 .. windows*ny exactly once, and the windows it treats as having ghost
// columns are those of the step kernel's edge test. Prints one line per
// failure and "share_cost ok <cases>" when all pass.
#include <cstdio>

#include "fv_internal.h"

int main() {
  using fvgb::ShareCost;
  const int nxs[] = {8, 27, 29, 30, 31, 32, 55, 56, 57, 64, 100, 300, 1023, 2048, 4096, 16384};
  const int nys[] = {5, 8, 37, 61, 130, 1024, 2048};
  const long long gs[] = {1, 2, 3, 7, 28, 64, 608, 2432, 4864, 29184};
  long long cases = 0, bad = 0;
  for (int nx : nxs) {
    for (int ny : nys) {
      const ShareCost sc(nx, ny);
      const long long windows = (nx + fvgb::kWarpCols - 1) / fvgb::kWarpCols;
      if (sc.windows != windows) {
        std::printf("windows nx=%d: %lld != %lld\n", nx, sc.windows, windows);
        ++bad;
      }
      for (long long w = 0; w < windows; ++w) {
        const long long xw = w * fvgb::kWarpCols;
        const bool edge = (xw - fvgb::kHalo <= 1) || (xw + fvgb::kLanes - fvgb::kHalo - 1 >= nx - 2);
        const bool model = (w == 0) || (w >= sc.w_hi1);
        if (edge != model) {
          std::printf("edge nx=%d w=%lld: kernel %d model %d\n", nx, w, (int)edge, (int)model);
          ++bad;
        }
      }
      const long long C = sc.total();
      for (long long G : gs) {
        ++cases;
        long long prev = 0;
        for (long long g = 0; g < G; ++g) {
          const long long s0 = sc.pos(g * C / G), s1 = sc.pos((g + 1) * C / G);
          if (s0 != prev || s1 < s0) {
            std::printf("tiling nx=%d ny=%d G=%lld g=%lld: [%lld, %lld) after %lld\n", nx, ny, G, g, s0, s1, prev);
            ++bad;
            break;
          }
          prev = s1;
        }
        if (prev != windows * ny) {
          std::printf("cover nx=%d ny=%d G=%lld: %lld of %lld\n", nx, ny, G, prev, windows * ny);
          ++bad;
        }
      }
    }
  }
  if (bad) return 1;
  std::printf("share_cost ok %lld\n", cases);
  return 0;
}
