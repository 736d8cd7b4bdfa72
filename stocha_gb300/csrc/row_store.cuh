// Row-major path output in whole 32-byte sectors.
//
// The materialised path arrays are C-order (n_paths, steps+1[, n_assets]) as
// the reference returns them (lib.rs:58-72), and one thread owns one row.  A
// plain per-step store from each lane writes 8 (or 4) bytes into 32 different
// rows, 2 KB apart: every DRAM sector is filled by four (eight) stores that
// come microseconds apart, and L2 evicts most of them part-written, so DRAM
// reads the sector back to merge it (measured: 1.5x the algorithmic bytes).
//
// RowStore stages each lane's values in shared memory and writes a sector only
// when it is complete, as one 32-byte vector store.  The first and last
// sectors of a row are shared with its neighbours: at the end of a row, lane l
// merges its last sector with the first elements of lane l+1's row (the next
// row) and writes it whole.  Only a sector whose neighbour row is not in the
// same warp (the launch's first or last row, or a launch whose base is not
// sector-aligned) is written element by element.
//
// Staging layout (per warp, lane-minor so that every access is conflict-free):
//   slot q of lane L at stage[q * 32 + L]: a ring of 2 sectors (q < 2 SE) and,
//   after it, the lane's head (q in [2 SE, 3 SE)): the row's elements that
//   share the first sector with the previous row.  3 KB per warp.
// Sector-relative offset o = ph + j of the row's element j, where ph is the
// row's offset in its first sector; element j lives in ring slot o mod 2 SE.
// Every SE puts the writer flushes the one sector completed since the last
// flush.  In the per-path loop kernels every lane of the warp makes the same
// put at once (whatever the number of values per step), so the sector stores
// of all lanes issue together; in the warp-uniform kernels each lane puts as
// its own steps complete, and its ring and writes are its own.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace stocha {

__device__ __forceinline__ void st_sector(double* p, const double* v) {
  asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p), "d"(v[0]), "d"(v[1]), "d"(v[2]), "d"(v[3])
               : "memory");
}
__device__ __forceinline__ void st_sector(float* p, const float* v) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(v[0]), "f"(v[1]),
               "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
               : "memory");
}

template <typename T>
struct RowStore {
  static constexpr uint32_t SE = 32 / sizeof(T);  // elements per sector
  static constexpr uint32_t RING = 2 * SE;        // ring slots
  static constexpr uint32_t SLOTS = RING + SE;    // ring + head
  T* stage;     // this lane's slot 0 (stride 32 elements between slots)
  T* base;      // the row's first sector (row - ph, sector-aligned)
  uint32_t ph;  // the row's offset in its first sector
  uint32_t o;   // sector-relative offset of the next element

  // Shared-memory bytes a block of `threads` threads needs.
  static constexpr uint32_t bytes(uint32_t threads) { return threads / 32 * SLOTS * 32 * (uint32_t)sizeof(T); }

  // smem: the block's staging area (bytes(blockDim.x)).
  __device__ __forceinline__ void init(T* smem) {
    stage = smem + (threadIdx.x >> 5) * SLOTS * 32 + (threadIdx.x & 31u);
  }
  __device__ __forceinline__ T& slot(uint32_t q) const { return stage[q * 32]; }

  __device__ __forceinline__ void begin(T* row) {
    ph = (uint32_t)(((uintptr_t)row / sizeof(T)) & (SE - 1));
    base = row - ph;
    o = ph;
  }

  // Writes the sector [s, s + SE); the row's first sector, when it is shared
  // (s == 0 < ph), moves to the head slots instead, for end().
  __device__ __forceinline__ void write(uint32_t s) {
    const uint32_t q0 = s & (RING - 1);
    if (s >= ph) {
      T v[SE];
#pragma unroll
      for (uint32_t k = 0; k < SE; ++k) v[k] = slot(q0 + k);
      st_sector(base + s, v);
    } else {
#pragma unroll 1
      for (uint32_t k = ph; k < SE; ++k) slot(RING + k) = slot(q0 + k);
    }
  }

  // Every SE puts of this lane exactly one sector boundary has been crossed
  // since its last write: write that sector.
  __device__ __forceinline__ void put(T v) {
    slot(o & (RING - 1)) = v;
    ++o;
    if (((o - ph) & (SE - 1)) == 0) write((o & ~(SE - 1)) - SE);
  }

  // Ends the row.  Called by all 32 lanes of the warp together; `on`: this
  // lane wrote a row; `next_on`: lane + 1 wrote the next row (row + 1).
  // Requires rows of at least 2 * SE elements (the first and last sectors of
  // a row are then distinct).
  __device__ __forceinline__ void end(bool on, bool next_on) {
    const uint32_t lane = threadIdx.x & 31u;
    if (on) {
      // a sector completed since the last write (at most one: writes come
      // every SE puts)
      const uint32_t last = o - ((o - ph) & (SE - 1));  // offset at the last write
      if ((o & ~(SE - 1)) > (last & ~(SE - 1))) write((o & ~(SE - 1)) - SE);
    }
    __syncwarp();
    if (on) {
      const uint32_t t = o & (SE - 1);  // this row's elements in its last sector
      if (t) {
        const uint32_t ls = o - t, q0 = ls & (RING - 1);
        if (next_on && lane < 31u) {  // lane + 1's row starts in this sector at offset t
          T v[SE];
          const T* nxt = stage + 1;
#pragma unroll
          for (uint32_t k = 0; k < SE; ++k) v[k] = k < t ? slot(q0 + k) : nxt[(RING + k) * 32];
          st_sector(base + ls, v);
        } else {
#pragma unroll 1
          for (uint32_t k = 0; k < t; ++k) base[ls + k] = slot(q0 + k);
        }
      }
      if (ph && lane == 0) {  // no previous row in this warp to merge with
#pragma unroll 1
        for (uint32_t k = ph; k < SE; ++k) base[k] = slot(RING + k);
      }
    }
    __syncwarp();
  }
};

// Store modes of the path kernels: fused (payoff sums, no path output),
// element stores (time-major columns, terminal values, short rows), or
// row-major rows through the staged sector writer.
enum : int { kFused = 0, kElems = 1, kRows = 2 };

// Path output of a kernel in mode kMode: the staged writer in kRows, nothing
// otherwise (the element stores address the output directly).
template <typename T, int kMode>
struct PathOut {
  RowStore<T> rs;
  // smem: RowStore<T>::bytes(blockDim.x) bytes of dynamic shared memory
  __device__ __forceinline__ void init(void* smem) {
    if (kMode == kRows) rs.init(reinterpret_cast<T*>(smem));
  }
  __device__ __forceinline__ void begin(T* row) {
    if (kMode == kRows) rs.begin(row);
  }
};

// Calls body(lrow) for this thread's rows (grid-stride over [0, rows)).  In
// the kRows mode the loop runs warp-uniformly, so that all 32 lanes end each
// row together (RowStore::end merges neighbouring rows across lanes).
template <typename T, int kMode, class Body>
__device__ __forceinline__ void for_rows(uint64_t rows, PathOut<T, kMode>& out, Body&& body) {
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  if constexpr (kMode != kRows) {
    for (uint64_t lrow = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; lrow < rows; lrow += nthreads) body(lrow);
  } else {
    for (uint64_t wb = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wb < rows; wb += nthreads) {
      const uint64_t lrow = wb + (threadIdx.x & 31u);
      const bool on = lrow < rows;
      if (on) body(lrow);
      out.rs.end(on, lrow + 1 < rows);
    }
  }
}

// The same rows for the warp-uniform kernels: body(lrow, on) is called by all
// 32 lanes of each warp (on: the lane has a row; lrow is then its row, else
// the warp's first row), because the sampler feed inside votes across the
// warp.  The loop runs warp-uniformly in every mode.
template <typename T, int kMode, class Body>
__device__ __forceinline__ void for_rows_warp(uint64_t rows, PathOut<T, kMode>& out, Body&& body) {
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t wb = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wb < rows; wb += nthreads) {
    const uint64_t lrow = wb + (threadIdx.x & 31u);
    const bool on = lrow < rows;
    body(on ? lrow : wb, on);
    if constexpr (kMode == kRows) out.rs.end(on, lrow + 1 < rows);
  }
}

}  // namespace stocha
