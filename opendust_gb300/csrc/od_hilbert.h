// od_hilbert.h — cell order of the cutoff path's sort: the index of a cell along a 3-D
// Hilbert curve. Plain C so that the host tests compile the same code the kernels run.
#ifndef OD_HILBERT_H
#define OD_HILBERT_H
#include <stdint.h>

#ifdef __CUDACC__
#define OD_HD __host__ __device__ __forceinline__
#else
#define OD_HD static inline
#endif

// Index of cell (x, y, z), each < 2^bits (1 <= bits <= 10), along a Hilbert curve through the
// 2^bits-sided grid: J. Skilling's transpose method ("Programming the Hilbert curve", AIP
// Conf. Proc. 707, 381 (2004)) — undo the excess work of the axes from the top bit down,
// Gray-encode, then interleave the transposed bits, x highest. Consecutive indices are
// face-adjacent cells, so runs of consecutive cells stay compact (a Morton order jumps across
// the grid at its block boundaries).
OD_HD uint32_t od_hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits) {
  uint32_t X[3] = {x, y, z};
  const uint32_t M = 1u << (bits - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; i++) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  X[2] ^= X[1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  X[0] ^= t;
  X[1] ^= t;
  X[2] ^= t;
  uint32_t key = 0;
  for (int b = bits - 1; b >= 0; b--)
    key = (key << 3) | (((X[0] >> b) & 1u) << 2) | (((X[1] >> b) & 1u) << 1) | ((X[2] >> b) & 1u);
  return key;
}

#endif
