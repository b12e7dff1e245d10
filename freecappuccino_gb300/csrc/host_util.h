// Small host-side helpers shared by the C++ translation units of libfcgpu.so.
#pragma once

#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

namespace fcg {

// Runs f(i) for i in [0, n) on all host threads (contiguous chunks, so per-thread
// work keeps its memory locality).  Small ranges run inline.
template <class Fn>
void parallel_for(long long n, Fn &&f, long long serial_below = 1 << 15) {
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  if (n < serial_below || nt == 1) {
    for (long long i = 0; i < n; ++i) f(i);
    return;
  }
  nt = (unsigned)std::min<long long>(nt, (n + serial_below - 1) / serial_below);
  long long chunk = (n + nt - 1) / nt;
  std::vector<std::thread> pool;
  pool.reserve(nt);
  for (unsigned t = 0; t < nt; ++t) {
    long long b = (long long)t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([b, e, &f] {
      for (long long i = b; i < e; ++i) f(i);
    });
  }
  for (auto &th : pool) th.join();
}

// splitmix64 finaliser; the counter-based generator below hashes (seed, stream, i).
inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Uniform double in [0, 1) for counter i of (seed, stream): 53 random bits.
inline double uniform01(uint64_t seed, uint64_t stream, uint64_t i) {
  uint64_t key = splitmix64(seed * 0x9E3779B97F4A7C15ULL ^ splitmix64(stream + 0x632BE59BD9B4E019ULL));
  uint64_t r = splitmix64(key + i * 0xD1B54A32D192ED03ULL);
  return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace fcg
