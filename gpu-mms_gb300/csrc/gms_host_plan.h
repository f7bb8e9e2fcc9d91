// Host-side plans of the host-to-host sorts: how the input copy is cut into
// chunks, and how the last merge round is cut into parts whose final output
// prefix is copied out early.  Plain C++ (no CUDA), so the CPU tests compile
// and check them directly.
#pragma once

#include <algorithm>
#include <cstdint>

namespace gms {

constexpr int kHostChunks = 16;  // most input chunks of one host-to-host sort
constexpr int kMaxParts = 64;    // most parts of a last round

inline int64_t host_ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Input chunk boundaries (in base tiles) for a host-fed sort of `tiles` base
// tiles with fan-in k and `passes` merge rounds: a unit of k^q tiles, q the
// most early rounds (at most passes - 1) whose unit still leaves eight units
// of input; chunks rising 1, 1, 2, ..., c-1 units from the start, a plateau
// of chunks of at least c units (c about an eighth of the input, at most 5,
// the plateau chunks larger where the chunk count would exceed kHostChunks),
// and falling c-1, ..., 1 to the end, the remainder taking its place in the
// falling part.  A small first chunk lets the sort start after a short copy,
// small last ones leave little to sort after the last copy, and every
// interior boundary on a unit lets q merge rounds run chunk by chunk.
// Returns the chunk count and fills start[0..count] (start[count] = tiles).
inline int host_chunk_plan(int64_t tiles, int k, int passes, int64_t* start) {
  int64_t unit = 1;
  for (int q = 0; q < passes - 1 && unit * k * 8 <= tiles; ++q) unit *= k;
  const int64_t units = host_ceil_div(tiles, unit);
  const int64_t c = std::max<int64_t>(1, std::min<int64_t>(units / 8, 5));
  int64_t sizes[kHostChunks];
  int n = 0;
  sizes[n++] = 1;
  for (int64_t s = 1; s < c; ++s) sizes[n++] = s;  // 1, 1, 2, ..., c-1
  const int nfall = (int)(c - 1);                    // c-1, ..., 1
  const int64_t rem = units - (1 + c * (c - 1));     // both ramps hold 1 + c(c-1) units
  const int slots = kHostChunks - n - nfall - 1;
  const int64_t plateau = rem > 0 ? std::max<int64_t>(c, host_ceil_div(rem, (int64_t)slots)) : c;
  const int64_t full = rem / plateau, r = rem - full * plateau;
  for (int64_t i = 0; i < full; ++i) sizes[n++] = plateau;
  bool placed = r == 0;
  for (int64_t s = c - 1; s >= 1; --s) {
    if (!placed && r >= s) {
      sizes[n++] = r;
      placed = true;
    }
    sizes[n++] = s;
  }
  if (!placed) sizes[n++] = r;
  int64_t used = 0;
  start[0] = 0;
  for (int i = 0; i < n; ++i) {
    used += sizes[i];
    start[i + 1] = std::min(tiles, used * unit);
  }
  return n;
}

// End tiles of the parts of a last round of `tiles` tiles launched in up to
// `parts` pieces (at most kMaxParts): even pieces, or with `ramp` (and at
// least 3 parts and 64 tiles) a first piece of 1/32 of the tiles, a second of
// 1/16 and the rest even, so that the first final prefix is ready early.
// Returns the number of ends written (the last is `tiles`; ends may repeat
// where the pieces run out, and a repeated end is an empty piece).
inline int host_split_ends(int64_t tiles, int parts, bool ramp, int64_t* ends) {
  int np = 0;
  parts = std::max(1, std::min(parts, kMaxParts));
  if (ramp && parts >= 3 && tiles >= 64) {
    ends[np++] = host_ceil_div(tiles, 32);
    ends[np++] = ends[0] + host_ceil_div(tiles, 16);
    const int64_t rest = host_ceil_div(tiles - ends[1], (int64_t)(parts - 2));
    for (int64_t t1 = ends[1] + rest; np < parts; t1 += rest) ends[np++] = std::min(tiles, t1);
  } else {
    const int64_t per = host_ceil_div(tiles, (int64_t)parts);
    for (int64_t t1 = per; np < parts; t1 += per) ends[np++] = std::min(tiles, t1);
  }
  ends[np - 1] = tiles;
  return np;
}

}  // namespace gms
