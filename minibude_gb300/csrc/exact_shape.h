// exact_shape.h -- compile-time shape constants of the exact kernel, shared by its host code.
#pragma once
#include <cstddef>
#include <cstdint>

namespace bude {

constexpr int kStages = 4;       // shared-memory ring depth
constexpr int kRecF4 = 4;        // 16-byte words per protein record (64 bytes)
constexpr int kAtomAlign = 8;    // protein atoms are padded to a multiple of this (covers every unroll)
constexpr int kMaxThreads = 512; // launch bound: keeps the register budget at 128 per thread
// Blocks of at most kNarrowThreads run a second compilation of the kernel, bound to
// kNarrowBlocks blocks per SM: a budget of 170 registers per thread instead of 128 (12 warps per
// SM with more independent work each beat 16 warps on the 128-register budget).
constexpr int kNarrowThreads = 128;
constexpr int kNarrowBlocks = 3;

// Dynamic shared memory of exact_kernel<P, U> for a launch shape.
inline size_t exact_smem_bytes(int P, int wgsize, int tile, int split, int cluster) {
  size_t b = (size_t)kStages * tile * kRecF4 * 16 + kStages * sizeof(uint64_t);
  if (split > 1 && cluster) b += (size_t)P * wgsize * sizeof(float);
  return b;
}

} // namespace bude
