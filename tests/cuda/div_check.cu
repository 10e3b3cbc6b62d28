// Checks div_rcp (Markstein quotient from a correctly rounded reciprocal, used by
// the collision kernel) against IEEE division __fdiv_rn, bit for bit.
//   sweep 1: every significand of a in [1, 2) against 4096 random b in [0.3, 3]
//   sweep 2: 2^30 random (a, b): |a| in [2^-60, 2^60], b in [2^-14, 2^14], random signs
// Prints "<mismatches> <cases>" and exits 0; every index is bounded by its loop.
#include <cstdio>
#include <cstdint>
#include "wt_lattice.cuh"

__device__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}

__global__ void sweep_significands(const float* bs, uint32_t nb, unsigned long long* bad) {
  const uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long local = 0;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < (1u << 23); t += stride) {
    const float a = __uint_as_float(0x3f800000u | t);
    for (uint32_t k = 0; k < nb; k++) {
      const float b = bs[k];
      const float r = __frcp_rn(b);
      local += (__float_as_uint(wt::div_rcp(a, b, r)) != __float_as_uint(__fdiv_rn(a, b)));
    }
  }
  atomicAdd(bad, local);
}

__global__ void sweep_random(uint32_t n, uint32_t seed, unsigned long long* bad) {
  const uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long local = 0;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const uint32_t h1 = hash32(t * 2u + seed), h2 = hash32(t * 2u + 1u + seed * 7919u);
    const uint32_t ea = 127u - 60u + (h1 >> 23) % 121u;   // 2^-60 .. 2^60
    const uint32_t eb = 127u - 14u + (h2 >> 23) % 29u;    // 2^-14 .. 2^14
    const float a = __uint_as_float(((h1 & 1u) << 31) | (ea << 23) | (h1 & 0x7fffffu));
    const float b = __uint_as_float((eb << 23) | (h2 & 0x7fffffu));
    const float r = __frcp_rn(b);
    local += (__float_as_uint(wt::div_rcp(a, b, r)) != __float_as_uint(__fdiv_rn(a, b)));
  }
  atomicAdd(bad, local);
}

int main() {
  const uint32_t nb = 4096;
  float hb[nb];
  uint32_t s = 12345u;
  for (uint32_t k = 0; k < nb; k++) {
    s = s * 1664525u + 1013904223u;
    hb[k] = 0.3f + 2.7f * (float)(s >> 8) * (1.0f / 16777216.0f);
  }
  float* db = nullptr;
  unsigned long long* dbad = nullptr;
  if (cudaMalloc(&db, sizeof(hb)) != cudaSuccess || cudaMalloc(&dbad, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemcpy(db, hb, sizeof(hb), cudaMemcpyHostToDevice);
  cudaMemset(dbad, 0, 2 * sizeof(unsigned long long));
  sweep_significands<<<1216, 256>>>(db, nb, dbad);
  sweep_random<<<1216, 256>>>(1u << 30, 77u, dbad + 1);
  unsigned long long hbad[2] = {0, 0};
  if (cudaMemcpy(hbad, dbad, sizeof(hbad), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  printf("%llu %llu\n", hbad[0] + hbad[1], (unsigned long long)nb * (1ull << 23) + (1ull << 30));
  cudaFree(db);
  cudaFree(dbad);
  return 0;
}
