// Device-side tile generation from a TileGen descriptor (see engine.h).
#pragma once
#include "common.cuh"
#include "engine.h"

namespace htgb {

HT_DEV Tile gen_tile(const TileGen &g, int idx) {
  Tile t;
  t.a_z = 0;
  t.b_row = 0;
  t.out_col = 0;
  if (g.kind == TILES_ROWS) {
    t.a_row = 128 * idx;
    t.out_row = 128ll * idx;
    t.valid_rows = static_cast<int>(min(128ll, g.rows - 128ll * idx));
    t.valid_cols = min(g.cols, g.bn);
  } else if (g.kind == TILES_SLABS) {
    const long long nlb = (g.L + 127) / 128;
    const long long r = idx / nlb, lb = idx - r * nlb;
    t.a_row = static_cast<int>(128 * lb);
    t.a_z = static_cast<int>(r);
    t.out_row = 128 * lb + g.L * r;
    t.valid_rows = static_cast<int>(min(128ll, g.L - 128 * lb));
    t.valid_cols = min(g.cols, g.bn);
  } else if (g.kind == TILES_GRID) {
    const long long nrb = (g.rows + g.bm - 1) / g.bm;
    const long long cb = idx / nrb, rb = idx - cb * nrb;
    t.a_row = static_cast<int>(g.bm * rb);
    t.b_row = static_cast<int>(g.bn * cb);
    t.out_row = g.bm * rb;
    t.out_col = static_cast<int>(g.bn * cb);
    t.valid_rows = static_cast<int>(min(static_cast<long long>(g.bm), g.rows - g.bm * rb));
    t.valid_cols = static_cast<int>(min(static_cast<long long>(g.bn), g.n - g.bn * cb));
  } else {
    int i = 0;
    while (i + 1 < g.ni && g.prefix[i + 1] <= idx) ++i;
    const int j = g.jmin[i] + (idx - g.prefix[i]);
    t.a_row = g.bm * i;
    t.b_row = g.bn * j;
    t.out_row = static_cast<long long>(g.bm) * i;
    t.out_col = g.bn * j;
    t.valid_rows = static_cast<int>(min(static_cast<long long>(g.bm), g.n - static_cast<long long>(g.bm) * i));
    t.valid_cols = static_cast<int>(min(static_cast<long long>(g.bn), g.n - static_cast<long long>(g.bn) * j));
  }
  return t;
}

}  // namespace htgb
