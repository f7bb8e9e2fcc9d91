// testmm: command-line driver with the reference's interface and output.
//
// Same usage and output lines as GPU-MMS's ./testMM (src/testMM.cu:49-63,
// 134-218), so its sweep scripts (scripts/allSizes.sh, raceConditions.sh, ...)
// run unchanged against this library:
//   usage   testmm <N> [ITERS]
//   input   srand(0); N keys rand()%1024, two rand() draws per key
//           (create_random_list, src/buildData.h:54-65)
//   timing  cudaEvents around multimergesort<int,cmp>(d_data, d_output, h_data, N)
//           including its synchronize; prints "avg min max" in ms over ITERS
//           calls (the reference's compile-time ITERS, default 1), each on a
//           fresh copy of the input (copied outside the events)
//   check   "SORTED!" or "NOT SORTED! Item at index i is less than its
//           predecessor." -- here SORTED! also requires the output to be a
//           permutation of the input (the reference checks order only)
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "multimergesort.hxx"

int main(int argc, char** argv) {
  if (argc != 2 && argc != 3) {
    printf("Usage: ./testMM <N>\n");
    exit(1);
  }
  const int N = atoi(argv[1]);
  const int iters = argc == 3 ? std::max(1, atoi(argv[2])) : 1;
  std::vector<int> h_data(N > 0 ? N : 1);
  srand(0);
  for (int i = 0; i < N; ++i) {
    h_data[i] = rand() % 1024;
    (void)rand();  // the second draw only reaches the upper half of a 64-bit DATATYPE
  }
  std::vector<int> input(h_data.begin(), h_data.begin() + N);
  int *d_data = nullptr, *d_output = nullptr;
  cudaMalloc(&d_data, sizeof(int) * (N > 0 ? N : 1));
  cudaMalloc(&d_output, sizeof(int) * (N > 0 ? N : 1));
  cudaEvent_t start, stop;
  cudaEventCreate(&start);
  cudaEventCreate(&stop);
  int* res = nullptr;
  double sum = 0, lo = 1e30, hi = 0;
  for (int it = 0; it < iters; ++it) {
    cudaMemcpy(d_data, h_data.data(), sizeof(int) * N, cudaMemcpyHostToDevice);
    cudaDeviceSynchronize();
    cudaEventRecord(start, 0);
    res = multimergesort<int, cmp<int>>(d_data, d_output, h_data.data(), N);
    cudaDeviceSynchronize();
    cudaEventRecord(stop, 0);
    cudaEventSynchronize(stop);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, start, stop);
    sum += ms;
    lo = std::min(lo, (double)ms);
    hi = std::max(hi, (double)ms);
  }
  printf("%lf %lf %lf\n", sum / iters, lo, hi);
  if (!res) res = d_output;
  cudaMemcpy(h_data.data(), res, sizeof(int) * N, cudaMemcpyDeviceToHost);
  int bad = -1;
  for (int i = 1; i < N; ++i) {
    if (host_cmp(h_data[i], h_data[i - 1])) {
      bad = i;
      break;
    }
  }
  if (bad < 0) {
    std::sort(input.begin(), input.end());
    for (int i = 0; i < N; ++i) {
      if (input[i] != h_data[i]) {
        bad = i;
        break;
      }
    }
  }
  if (bad >= 0)
    printf("NOT SORTED! Item at index %d is less than its predecessor.\n", bad);
  else
    printf("SORTED!\n");
  cudaFree(d_data);
  cudaFree(d_output);
  return 0;
}
