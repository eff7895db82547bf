// The code that describes, prepares and launches one kernel variant (a Cfg). Each
// compilation of gqs_variant_tu.cu instantiates it for one entry of gqs_variant_table.h.
#pragma once
#include "gqs_device.cuh"
#include "gqs_launch.h"

namespace gqs {

template <class C>
struct VariantOps {
  static VariantInfo info(const char* name) {
    VariantInfo vi;
    vi.ncw = C::NCW;
    vi.threads = C::NT;
    vi.tile = C::TILE;
    vi.chunk = C::CHUNK;
    vi.kpt = C::KPT;
    vi.stages = C::STAGES;
    vi.tiny = C::TINY;
    vi.smem = sizeof(Smem<C>);
    vi.name = name;
    return vi;
  }
  static int prepare() {
    const size_t smem = sizeof(Smem<C>);
    if (cudaFuncSetAttribute(persistent_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return 0;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, persistent_kernel<C>, C::NT, smem) != cudaSuccess)
      return 0;
    return blocks;
  }
  static cudaError_t launch(const LaunchParams& p) {
    using B = typename C::B;
    SortArgs<typename C::T> a;
    a.d = static_cast<B*>(p.d);
    a.dn = static_cast<B*>(p.dn);
    a.jobs = p.jobs;
    a.q = p.q;
    a.tmap = p.tmap;
    a.capacity = p.capacity;
    a.tmask = p.tmask;
    a.timeout_ns = p.timeout_ns;
    a.n = p.check_n ? p.check_n : p.n;
    const uint32_t nseg = p.offsets ? p.nseg : 1u;
    const uint32_t seed_blocks = (nseg + 7u) / 8u;  // 8 warps per 256-thread block, one per segment
    // After a top split the seed kernel follows split_scatter as a programmatic dependent
    // launch; the persistent kernel follows the seed kernel so whenever no event lies between.
    cudaError_t e = launch_kernel(p.from_dn != 0, seed_kernel<C>, dim3(seed_blocks), dim3(256), 0, p.stream, a,
                                  p.offsets, p.nseg_dev, nseg, (unsigned long long)p.n, p.pairs, p.from_dn);
    if (e != cudaSuccess) return e;
    if (p.ev_begin) cudaEventRecord(p.ev_begin, p.stream);
    e = launch_kernel(p.ev_begin == nullptr, persistent_kernel<C>, dim3(p.grid), dim3(C::NT), sizeof(Smem<C>),
                      p.stream, a);
    if (p.ev_end) cudaEventRecord(p.ev_end, p.stream);
    return e;
  }
};

}  // namespace gqs
