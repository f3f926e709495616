// vf_tma.cuh -- tensor-memory-accelerator (TMA) staging of tiles.
//
// The Float64 tile kernels stage each tile of the state (w, hu, hv planes), of
// the stage-1 derivative and friction factor, and of the bottom corners into
// shared memory with one cp.async.bulk.tensor per array, issued by one thread
// and completed on an mbarrier; the other threads never compute an address.
// Tensor maps describe the padded device layout (rows of pitch P elements with
// XOFF leading pad columns, planes PS elements apart); coordinates past the
// last column or row read as zero, which is what the plain loads give there.
//
// Alignment rules the kernels check before issuing a copy: the innermost
// coordinate times the element size is a multiple of 16 bytes (the tiles start
// at even columns of Float64 rows), and the shared-memory destination is
// 128-byte aligned. A block that cannot use TMA loads its tile the plain way.
// The stage pass also writes its output tile (the interior cells; ghost cells
// are written with plain stores) from shared memory with one tensor store.
// Out-of-range clipping of a store is not exact to the element along x: with
// the extent ending inside a 16-byte chunk, the store also wrote the rest of
// that chunk (the first ghost column of a grid with an odd interior width,
// measured on GB300). So the store maps' x extent ends at a 32-byte multiple
// at or below the last interior column (tma_store_cols), and the interior
// columns past it are written with plain stores; no tensor store reaches a
// ghost cell or padding.
// Waits are bounded: a wait that gives up records the fact in the step record
// and the block loads its tile the plain way.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace vf {

// Tensor maps of one handle's buffers (Float64 tile kernels only). A launch
// uses them only when its buffers are the ones the maps were made for.
struct TmaMaps {
  CUtensorMap U[2];  // the two state volumes: 3D (x, y, plane), box HX x HY x 3
  CUtensorMap Ust[2];  // the same volumes for tile stores: interior extent only, box TX x TY x 3
  CUtensorMap L;     // stage-1 derivative planes, same shape
  CUtensorMap S;     // friction factor, 2D, box HX x HY
  CUtensorMap B;     // bottom corners, 2D, box BHX x BHY
  const void* Ub[2];
  const void* Lb;
  const void* Sb;
  const void* Bb;
  int ok;
};

// x extent (in 8-byte elements, from the row start) of a tile-store map for
// rows whose interior ends before column `cols`: rounded down to 32 bytes.
#if defined(__CUDACC__)
__host__ __device__
#endif
    inline int tma_store_cols(int cols) {
  return cols & ~3;
}

#if defined(__CUDACC__)

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wall-clock limit of one tile-copy wait. A tile copy completes in
// microseconds; a wait that runs this long has lost its copy. (Kept well
// above a preemption time slice, so a block that is merely descheduled does
// not give up; a block that gives up waits once more before it exits, so a
// lost copy costs it at most twice this.)
constexpr unsigned long long kTileWaitLimitNs = 50000000ull;  // 50 ms

// Bounded wait for the phase to complete: gives up after `limit` polls or
// after kTileWaitLimitNs of wall clock (%globaltimer), whichever comes first
// (each try_wait may suspend the thread for a short, hardware-bounded time);
// false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned phase, int limit = 1 << 22) {
  const unsigned long long t0 = globaltimer_ns();
  for (int i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, phase)) return true;
    if ((i & 63) == 63 && globaltimer_ns() - t0 > kTileWaitLimitNs) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

// Shared -> global tile store (bulk group). Elements outside the map's extent
// are not written. The source must be made visible to the async proxy first
// (fence_async_smem by the writing threads, then a block barrier).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int c0, int c1, int c2) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(smem_addr(src)), "r"(c0), "r"(c1), "r"(c2)
               : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Waits until this thread's committed bulk stores have completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// The copy rules this file relies on: x * element size a multiple of 16 bytes,
// destination 128-byte aligned.
__device__ __forceinline__ bool tma_ok(int x, int elem, const void* dst) {
  return ((x * elem) & 15) == 0 && (smem_addr(dst) & 127) == 0;
}

#endif  // __CUDACC__

}  // namespace vf
