/*
 * cmp.hxx -- the datatype / comparator plugin surface, GB300 build.
 *
 * Same names and meaning as the reference's plugin file (GPU-MMS
 * src/cmp.hxx:21-54):
 *   DATATYPE   the key type the default instantiation sorts
 *   CASTTYPE   kept for source compatibility (the reference shuffles keys as
 *              CASTTYPE; this implementation never shuffles keys, so any
 *              copyable type works)
 *   MAXVAL / MINVAL  kept for source compatibility; NOT reserved: every key
 *              value, including MAXVAL, sorts correctly here
 *   fptr_t     int(*)(DATATYPE, DATATYPE)
 *   cmp<T>     device strict weak order, default a < b
 *   host_cmp<T> its host twin
 * Every definition is guarded, so a project can supply its own before
 * including this file.  multimergesort<T, f> accepts any
 * `__device__ int f(T, T)` strict weak order, for any T (several types per
 * translation unit are fine).
 */
#ifndef GMS_CMP_HXX_
#define GMS_CMP_HXX_

#ifndef DATATYPE
#define DATATYPE int
#endif
#ifndef CASTTYPE
#define CASTTYPE int
#endif
#ifndef MAXVAL
#define MAXVAL 2147483647
#endif
#ifndef MINVAL
#define MINVAL -2147483647
#endif

typedef int (*fptr_t)(DATATYPE, DATATYPE);

#ifndef GMS_USER_CMP
template <typename T>
__forceinline__ __device__ int cmp(T a, T b) {
  return a < b;
}
template <typename T>
__forceinline__ int host_cmp(T a, T b) {
  return a < b;
}
#endif

#endif /* GMS_CMP_HXX_ */
