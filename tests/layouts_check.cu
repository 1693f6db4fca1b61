// Host-side checks of the layout arithmetic the training kernels rely on (run on the CPU by
// tests/test_layouts.py): a row-tiled [rows][128] tile is byte for byte the MN-major operand tile
// the weight-gradient UMMAs read (so it can arrive as one bulk copy), the MN-major tiles are
// one-to-one over their bytes, and the gradient reduction's transposition puts column-major
// partials back row-major.
#include <cstdio>
#include <vector>

#include "wgrad_tc.cuh"

using namespace bude;

int main() {
  int bad = 0;
  for (int r = 0; r < 128; ++r)
    for (int k = 0; k < kHid; ++k)
      if (kmajor_offset(r, k, kHid) != mnmajor_offset(k, r, kHid)) ++bad;
  for (long long row : {0LL, 1LL, 127LL, 128LL, 1000LL, 327679LL})
    for (int k : {0, 7, 8, 127})
      if (tiled_offset(row, k, kHid) != (row / 128) * (long long)kWgZ + kmajor_offset((int)(row % 128), k, kHid)) ++bad;
  for (int nmn : {kHid, kWgN1, kWgNb}) {
    std::vector<char> seen(wg_tile_bytes(nmn), 0);
    for (int mn = 0; mn < nmn; ++mn)
      for (int k = 0; k < kWgTile; ++k) {
        const uint32_t off = mnmajor_offset(mn, k, nmn);
        if (off % 2 || off >= seen.size() || seen[off]) {
          ++bad;
          continue;
        }
        seen[off] = 1;
      }
  }
  for (int cols : {kHid, kFeat, kMaxTypes})
    for (int c = 0; c < cols; ++c)
      for (int m = 0; m < kHid; ++m)
        if (reduce_dst_index(c * kHid + m, kHid, cols) != m * cols + c) ++bad;
  if (reduce_dst_index(5, 0, 0) != 5) ++bad;
  // slots: 128-byte aligned, inside the region, not overlapping
  const uint32_t starts[] = {kWgSlot3, kWgSlot2, kWgSlot1, kWgSlot4, kWgOnes, kWgRegion};
  for (int i = 0; i + 1 < 6; ++i)
    if (starts[i] % 128 || starts[i + 1] <= starts[i]) ++bad;
  if (kWgSlot2 - kWgSlot3 != 2 * kWgZ || kWgSlot1 - kWgSlot2 != 2 * kWgZ ||
      kWgSlot4 - kWgSlot1 != kWgZ + wg_tile_bytes(kWgN1) || kWgOnes - kWgSlot4 != kWgZ + wg_tile_bytes(kWgNb) ||
      kWgRegion - kWgOnes != wg_tile_bytes(kWgNb))
    ++bad;
  std::printf(bad ? "FAIL %d\n" : "ok\n", bad);
  return bad != 0;
}
