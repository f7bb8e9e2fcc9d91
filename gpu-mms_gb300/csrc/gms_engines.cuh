// Engines of the prebuilt dtypes, shared by the C ABI (libgms.so) and the
// header-only drop-in (include/multimergesort.hxx), which instantiates the
// same keys-only engine in the caller's translation unit for built-in integer
// keys under the default comparator.
#pragma once

#include <cstdint>
#include <type_traits>

#include "gms_sort.cuh"

namespace gms_engines {

// Item counts per thread are odd, so the thread-strided shared-memory
// accesses of a warp fall in distinct banks.  Geometries were chosen by
// timing on GB300 (2^28 int32 keys, 2^27 uint64 keys, 2^27 uint64 / float32
// keys with int32 payload):
//   keys only   base: warp-shuffle base case (8192-key tiles for 32-bit
//               keys, 4096 for 64-bit keys); 512 x 17 for tile_sort; data
//               rounds with one merge stream per window and runs padded with
//               sentinels: 288 x 31 (32-bit keys: three CTAs of ~76 KB shared
//               memory per SM) or 256 x 17 (64-bit keys)
//   key/value   base 256 x 17, data rounds 288 x 15 (keys + payload staged)
//   index rounds (a block sample merged with its uint32 positions) 256 x 17,
//               512 x 17 for 32-bit keys-only sorts
constexpr int kNT = 512;
constexpr int kItems = 17;
using IndexGeo = gms::MergeGeo<256, 17>;
template <class Key>
using KeysGeo = std::conditional_t<sizeof(Key) == 4, gms::MergeGeo<288, 31, 1>, gms::MergeGeo<256, 17, 1>>;
// keys-only 32-bit sorts: index rounds of 512 x 17, so a first-round group's
// block sample (32 runs x 256 entries) is merged by one CTA
template <class Key>
using KeysIndexGeo = std::conditional_t<sizeof(Key) == 4, gms::MergeGeo<512, 17>, IndexGeo>;

// (parameter names avoid the reference's single-letter macros of params.h,
// which callers of the drop-in header include first)
template <class Key, class Codec>
using KeysEngine =
    gms::Engine<Key, gms::NoVal, gms::KeyLess, Codec, false, kNT, kItems, KeysGeo<Key>, KeysIndexGeo<Key>>;
// key/value data rounds: 288 x 15, one merge stream per window (uint64 keys +
// int32 payload, 2^27: merge rounds 6.63 ms against 7.41 for 256 x 17 with two
// streams)
template <class Key, class Codec>
using KvEngine =
    gms::Engine<Key, int32_t, gms::KeyLess, Codec, true, 256, 17, gms::MergeGeo<288, 15, 1>, IndexGeo>;

// CTAs per SM the data-round merges are compiled for (their shared memory
// decides; see MergeMinBlocks): three for keys-only and float32 + int32
// rounds, two for uint64 + int32 rounds.
static_assert(gms::MergeMinBlocks<gms::MergeLayoutOf<uint32_t, gms::NoVal, gms::KeyLess, 288, 31, 1, false>>::value == 3,
              "32-bit keys-only merge: three CTAs per SM");
static_assert(gms::MergeMinBlocks<gms::MergeLayoutOf<uint64_t, gms::NoVal, gms::KeyLess, 256, 17, 1, true>>::value == 3,
              "64-bit keys-only merge (persistent): three CTAs per SM");
static_assert(gms::MergeMinBlocks<gms::MergeLayoutOf<uint32_t, int32_t, gms::KeyLess, 288, 15, 1, true>>::value == 3,
              "32-bit key/value merge (persistent): three CTAs per SM");
static_assert(gms::MergeMinBlocks<gms::MergeLayoutOf<uint64_t, int32_t, gms::KeyLess, 288, 15, 1, true>>::value == 2,
              "64-bit key/value merge (persistent): two CTAs per SM");

// Fan-in of a sort of n keys over base-case runs of `base` keys: a round
// costs about the same whatever its fan-in, so the sort takes the fewest
// rounds a fan-in of at most 32 allows, R = ceil(log2(runs) / 5), with the
// smallest power-of-two fan-in that still needs only R rounds,
// 2^ceil(log2(runs) / R) (int32 2^24: fan-in 16 in three even rounds, 0.49
// ms, against 32, 32, 2 with a fan-in of 32, 0.60 ms on GB300), and a block
// sample of 64 keys when that fan-in is below `wide_below` (keys-only sorts:
// 32; sorts with a payload, whose smaller tiles lose more to the coarser
// sample: 16).  Other tunables stay as in t.
inline gms::Tune balanced_fan_in(int64_t n, int64_t base, gms::Tune t, int wide_below = 32) {
  int lg = 0;  // log2 of the base-case runs, rounded up
  while ((base << lg) < n && lg < 40) ++lg;
  const int rounds = (lg + 4) / 5;
  if (rounds > 0) {
    t.k = 1 << ((lg + rounds - 1) / rounds);
    t.sample_b = t.k < wide_below ? 64 : 32;
  }
  return t;
}

// Built-in key types that sort through KeysEngine: the stored unsigned type
// and the codec that maps the key's order onto it.  Integers only: their
// equal keys are identical, so the keys-only (unstable) engine gives the same
// bits as a stable sort.
template <class T, class = void>
struct BuiltinKey {
  static constexpr bool value = false;
};
template <class T>
struct BuiltinKey<T, std::enable_if_t<std::is_integral<T>::value && (sizeof(T) == 4 || sizeof(T) == 8)>> {
  static constexpr bool value = true;
  using Stored = std::conditional_t<sizeof(T) == 4, uint32_t, uint64_t>;
  using Codec = std::conditional_t<std::is_signed<T>::value,
                                   std::conditional_t<sizeof(T) == 4, gms::SignFlip32, gms::SignFlip64>,
                                   gms::IdentityCodec<Stored>>;
};

}  // namespace gms_engines
