// Pins the CPU oracle to the reference's own code.  Built only where the
// GPU-MMS sources are present (see oracle/Makefile); the binary goes to
// oracle/_ref/ and never ships.  It includes the reference's test driver
// (src/testMM.cu) unchanged, renames its CLI entry point, and exposes three
// reference routines on the host:
//   create_random_list<int>  (src/buildData.h:54-65) after srand(seed)
//                            (src/testMM.cu:156)   -- the reference's input
//   selection_sort<int,host_cmp> (src/testMM.cu:308-320) over the whole
//                            array                 -- its CPU sort checker
//   the same selection sort per M-element tile plus the N%M tail, exactly as
//                            test_squareSort checks the base case
//                            (src/testMM.cu:264-269)
// Output: a binary file  int64 n | int32 input[n] | int32 sorted[n] |
//                        int32 tile_sorted[n]
#define main gms_reference_testmm_main
#include "testMM.cu"
#undef main

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: ref_pin <n> <seed> <out.bin>\n");
    return 2;
  }
  const int n = atoi(argv[1]);
  const unsigned seed = (unsigned)strtoul(argv[2], nullptr, 10);
  std::vector<int> in(n > 0 ? n : 1), full(n > 0 ? n : 1), tiles(n > 0 ? n : 1);
  srand(seed);
  create_random_list<int>(in.data(), n);
  full = in;
  selection_sort<int, host_cmp>(full.data(), n);
  tiles = in;
  int s = 0;
  for (; s <= n - M; s += M) selection_sort<int, host_cmp>(tiles.data() + s, M);
  selection_sort<int, host_cmp>(tiles.data() + s, n - s);
  FILE* f = fopen(argv[3], "wb");
  if (!f) return 3;
  long long nn = n;
  fwrite(&nn, sizeof(nn), 1, f);
  fwrite(in.data(), sizeof(int), n, f);
  fwrite(full.data(), sizeof(int), n, f);
  fwrite(tiles.data(), sizeof(int), n, f);
  fclose(f);
  return 0;
}
