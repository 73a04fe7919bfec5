// PCG32 (XSH-RR) as brisc's cyutils restates it (brisc/cyutils.pyx:1153-1177,
// 1228-1232): the generator behind the start vector of the PCA and the random
// k-means initialisation. Host code.
#pragma once

#include <stdint.h>

namespace bgpu {

inline uint32_t pcg_rand(uint64_t* state) {  // cyutils.pyx:1153-1158
  const uint64_t x = *state;
  *state = x * 6364136223846793005ULL + 1442695040888963407ULL;
  const uint32_t s = (uint32_t)((x ^ (x >> 18)) >> 27);
  const uint32_t rot = (uint32_t)(x >> 59);
  return (s >> rot) | (s << ((0u - rot) & 31u));
}

inline uint64_t pcg_srand(uint64_t seed) {  // cyutils.pyx:1228-1232
  uint64_t state = seed + 1442695040888963407ULL;
  pcg_rand(&state);
  return state;
}

// Lemire's bounded integer in [0, bound) (cyutils.pyx:1161-1172).
inline uint32_t pcg_randint(uint32_t bound, uint64_t* state) {
  uint64_t m = (uint64_t)pcg_rand(state) * (uint64_t)bound;
  uint32_t l = (uint32_t)m;
  if (l < bound) {
    const uint32_t threshold = (0u - bound) % bound;
    while (l < threshold) {
      m = (uint64_t)pcg_rand(state) * (uint64_t)bound;
      l = (uint32_t)m;
    }
  }
  return (uint32_t)(m >> 32);
}

inline float pcg_uniform(uint64_t* state) {  // cyutils.pyx:1175-1177
  return (float)pcg_rand(state) / (float)4294967295u;
}

}  // namespace bgpu
