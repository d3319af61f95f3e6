// Tensor-memory-accelerator (TMA) tile copies and mbarrier completion for
// sm_90+ (inline PTX), plus the host-side tensor-map encoder obtained from
// the driver through the runtime (no link against libcuda).
//
// Every wait on an mbarrier is bounded: a wait that runs out reports failure
// to its caller, which records an error status and leaves the kernel, so a
// copy that never completes cannot hang the GPU.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace osgpu {
namespace tma {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// One-thread initialisation of an mbarrier expecting `count` arrivals,
// made visible to the async proxy (the TMA unit) before any copy uses it.
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arrival of the issuing thread that also announces `bytes` of transactions.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with parity `parity` to complete: true when it
// did, false after `max_polls` polls (each try_wait suspends the thread for a
// hardware-chosen interval, so the bound is well beyond any real copy).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          unsigned max_polls = 1u << 22) {
  for (unsigned i = 0; i < max_polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 3-D tiled TMA load of one box at coordinates (c0, c1, c2) into shared
// memory, completing `bar` with the box's bytes.  c0 * element size must be a
// multiple of 16 bytes.
__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                        unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2),
      "r"(smem_u32(bar))
      : "memory");
}

// Untiled bulk copy of `bytes` contiguous bytes (16-byte aligned addresses,
// size a multiple of 16) from global into shared memory, completing `bar`.
__device__ __forceinline__ void load_bulk(void* dst, const void* src, unsigned bytes,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// 3-D tiled TMA store of one box from shared memory to coordinates
// (c0, c1, c2), tracked by the issuing thread's bulk-async group.  The
// writers of the box must have run fence_async_shared() and a barrier with
// the issuing thread first; coordinates are never negative, and c0 *
// element size is a multiple of 16 bytes.
__device__ __forceinline__ void store_3d(const CUtensorMap* map, const void* src, int c0, int c1,
                                         int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
          reinterpret_cast<unsigned long long>(map)),
      "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(src))
      : "memory");
}

// Close the issuing thread's current group of bulk stores.
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Until every committed store group of this thread has read its shared-memory
// source (the source may then be overwritten).
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Until every committed store group of this thread has completed its writes.
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Order this thread's generic-proxy shared-memory writes before later
// async-proxy (TMA) reads of them.
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<unsigned long long>(map))
               : "memory");
}

}  // namespace tma

// Host: encode a 3-D tiled tensor map of 8-byte elements (complex64) with
// dimensions dims[0..2] (dims[0] contiguous), byte strides of dimensions 1
// and 2, and box box[0..2].  Returns false when the driver entry point is
// unavailable or rejects the map (the caller then takes its non-TMA path).
bool encode_map_3d_c64(CUtensorMap* map, const void* base, const unsigned long long dims[3],
                       const unsigned long long strides[2], const unsigned box[3]);

}  // namespace osgpu
