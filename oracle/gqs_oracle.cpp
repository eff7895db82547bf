// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the GPU-Quicksort sort path.
//
// Nothing in the product library links, loads or calls this file. It is loaded
// by the test suite (as the parity checker), by __graft_entry__.smoke(), and
// by bench.py's CPU-baseline leg (timed as the reference's CPU path).
//
// Contents:
//   * oracle_gpuqsort_*  -- a CPU restatement of the reference's templated
//     GPUQSort<T> (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-906) with its
//     two kernels, gqsort_kernel (GPU-Quicksort_OpenCL_1.2/QuicksortKernels.cl:
//     102-240) and lqsort_kernel (QuicksortKernels.cl:267-421), emulated one
//     work-group at a time with the NVIDIA tuning constants
//     (GPU-Quicksort_Full_SYCL/Quicksort.h:124-129). Work-groups of one level
//     may run on several host threads; with threads == 1 every level runs its
//     blocks in block order, exactly as a serial device would.
//   * oracle_std_sort_*  -- std::sort, the reference's own verifier
//     (TRUST_BUT_VERIFY, GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:1120-1138).
//   * oracle_parallel_sort_* -- GCC parallel-mode sort on all cores, standing in
//     for the reference's tbb::parallel_sort (QuicksortMain.cpp:993), because
//     TBB is not installed.
//   * oracle_cpu_quicksort_* -- the reference's own CPU quicksort<T>
//     (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:213-259), which its main()
//     leaves commented out.
//
// Pinning: the reference cannot be built here (its path needs an OpenCL GPU
// platform and CL/cl.h, TBB, and DPC++ for the SYCL variants). The restatement
// is pinned by the reference's own known-answer test (a shuffled 1..N must come
// back as out[i] == i + 1, QuicksortMain.cpp:975-976) and by the reference's
// verifier, std::sort, on every committed golden vector.
//
// Deliberate difference: the Full-SYCL bitonic network compares through
// `uint av, bv` even for float and double (QuicksortMain.cpp:328-334,
// 342-345), which truncates non-integral keys. The restatement compares in T,
// as the OpenCL 1.2 kernels do for their uint keys.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#include <parallel/algorithm>
#include <omp.h>

namespace {

// Tuning constants, NVIDIA_GPU branch (GPU-Quicksort_Full_SYCL/Quicksort.h:124-129).
constexpr uint32_t QUICKSORT_BLOCK_SIZE = 1024;
constexpr uint32_t GQSORT_LOCAL_WORKGROUP_SIZE = 128;
constexpr uint32_t LQSORT_LOCAL_WORKGROUP_SIZE = 256;
constexpr uint32_t SORT_THRESHOLD = 512;
constexpr uint32_t EMPTY_RECORD = 42;  // Quicksort.h:139

// Median of three with the reference's tie rules (Quicksort.h:34-57).
template <class T>
T median(T x1, T x2, T x3) {
  if (x1 < x2) {
    if (x2 < x3) return x2;
    return (x1 < x3) ? x3 : x1;
  }
  if (x1 < x3) return x1;
  return (x2 < x3) ? x2 : x3;
}

// Records crossing the host/device boundary (Quicksort.h:145-184).
template <class T>
struct work_record {
  uint32_t start = 0, end = 0;
  T pivot = T(0);
  uint32_t direction = EMPTY_RECORD;
};
struct parent_record {
  uint32_t sstart, send, oldstart, oldend, blockcount;
};
template <class T>
struct block_record {
  uint32_t start, end;
  T pivot;
  uint32_t direction, parent;
};

// MAXSEQ heuristic (QuicksortMain.cpp:831-833).
size_t optp(size_t s, double k, size_t m) {
  return (size_t)std::pow(2.0, std::floor(std::log(s * k + m) / std::log(2.0) + 0.5));
}

// Exclusive prefix over work-item counts, as the up-sweep/down-sweep of
// QuicksortKernels.cl:150-173 leaves it; returns the total.
uint32_t exclusive_scan(uint32_t* v, uint32_t n) {
  uint32_t acc = 0;
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t c = v[i];
    v[i] = acc;
    acc += c;
  }
  return acc;
}

// One gqsort work-group (QuicksortKernels.cl:102-240).
template <class T>
void gqsort_block(T* d, T* dn, const block_record<T>& blk, parent_record* parents,
                  work_record<T>* news, size_t blockid) {
  const uint32_t WG = GQSORT_LOCAL_WORKGROUP_SIZE;
  T* s = blk.direction == 1 ? d : dn;
  T* sn = blk.direction == 1 ? dn : d;
  const T pivot = blk.pivot;
  uint32_t lt[WG], gt[WG];
  // Pass 1: each work-item counts its strided keys (lines 135-143).
  for (uint32_t l = 0; l < WG; ++l) {
    uint32_t ltp = 0, gtp = 0;
    for (uint32_t i = blk.start + l; i < blk.end; i += WG) {
      T tmp = s[i];
      if (tmp < pivot) ++ltp;
      if (tmp > pivot) ++gtp;
    }
    lt[l] = ltp;
    gt[l] = gtp;
  }
  uint32_t ltsum = exclusive_scan(lt, WG);
  uint32_t gtsum = exclusive_scan(gt, WG);
  // Reserve this block's output ranges in the parent (lines 183-186).
  parent_record& p = parents[blk.parent];
  uint32_t lbeg = __atomic_fetch_add(&p.sstart, ltsum, __ATOMIC_ACQ_REL);
  uint32_t gbeg = __atomic_fetch_sub(&p.send, gtsum, __ATOMIC_ACQ_REL) - gtsum;
  // Pass 2: scatter (lines 191-203).
  for (uint32_t l = 0; l < WG; ++l) {
    uint32_t lfrom = lbeg + lt[l], gfrom = gbeg + gt[l];
    for (uint32_t i = blk.start + l; i < blk.end; i += WG) {
      T tmp = s[i];
      if (tmp < pivot) sn[lfrom++] = tmp;
      if (tmp > pivot) sn[gfrom++] = tmp;
    }
  }
  // The last block of the parent fills the pivot run and writes the two
  // children with median-of-three pivots (lines 206-238).
  if (__atomic_fetch_sub(&p.blockcount, 1u, __ATOMIC_ACQ_REL) == 0) {
    uint32_t sstart = __atomic_load_n(&p.sstart, __ATOMIC_ACQUIRE);
    uint32_t send = __atomic_load_n(&p.send, __ATOMIC_ACQUIRE);
    uint32_t oldstart = p.oldstart, oldend = p.oldend;
    for (uint32_t i = sstart; i < send; ++i) d[i] = pivot;
    T lpivot = sn[oldstart];
    T gpivot = sn[oldend - 1];
    if (oldstart < sstart) lpivot = median(lpivot, sn[(oldstart + sstart) >> 1], sn[sstart - 1]);
    if (send < oldend) gpivot = median(sn[send], sn[(oldend + send) >> 1], gpivot);
    uint32_t direction = blk.direction ^ 1u;
    news[2 * blockid] = work_record<T>{oldstart, sstart, lpivot, direction};
    news[2 * blockid + 1] = work_record<T>{send, oldend, gpivot, direction};
  }
}

// Bitonic network over 2 * LQSORT_LOCAL_WORKGROUP_SIZE keys
// (QuicksortKernels.cl:40-68); each stage's pairs are disjoint, so visiting the
// work-items in order is the same as running them together.
template <class T>
void bitonic_sort(T* sh) {
  const uint32_t WG = LQSORT_LOCAL_WORKGROUP_SIZE;
  for (uint32_t ulevel = 1; ulevel < WG; ulevel <<= 1) {
    for (uint32_t j = ulevel; j > 0; j >>= 1) {
      for (uint32_t l = 0; l < WG; ++l) {
        uint32_t pos = 2 * l - (l & (j - 1));
        uint32_t direction = l & ulevel;
        T av = sh[pos], bv = sh[pos + j];
        bool sortThem = av > bv;
        T greater = sortThem ? av : bv;
        T lesser = sortThem ? bv : av;
        sh[pos] = direction ? greater : lesser;
        sh[pos + j] = direction ? lesser : greater;
      }
    }
  }
  for (uint32_t j = WG; j > 0; j >>= 1) {
    for (uint32_t l = 0; l < WG; ++l) {
      uint32_t pos = 2 * l - (l & (j - 1));
      T av = sh[pos], bv = sh[pos + j];
      bool sortThem = av > bv;
      sh[pos] = sortThem ? bv : av;
      sh[pos + j] = sortThem ? av : bv;
    }
  }
}

// Runs of at most SORT_THRESHOLD keys, padded with the type's maximum
// (QuicksortKernels.cl:70-97; GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:351-380).
template <class T>
void sort_threshold(T* data_in, T* data_out, uint32_t start, uint32_t end, T* temp) {
  uint32_t tsum = end - start;
  if (tsum == SORT_THRESHOLD) {
    bitonic_sort(data_in + start);
    for (uint32_t i = 0; i < SORT_THRESHOLD; ++i) data_out[start + i] = data_in[start + i];
  } else if (tsum > 1) {
    for (uint32_t i = 0; i < SORT_THRESHOLD; ++i)
      temp[i] = i < tsum ? data_in[start + i] : std::numeric_limits<T>::max();
    bitonic_sort(temp);
    for (uint32_t i = 0; i < tsum; ++i) data_out[start + i] = temp[i];
  } else if (tsum == 1) {
    data_out[start] = data_in[start];
  }
}

struct workstack_record {
  uint32_t start, end, direction;
};

// One lqsort work-group (QuicksortKernels.cl:267-421).
template <class T>
void lqsort_record(T* d, T* dn, const work_record<T>& block) {
  const uint32_t WG = LQSORT_LOCAL_WORKGROUP_SIZE;
  std::vector<T> mys(QUICKSORT_BLOCK_SIZE), mysn(QUICKSORT_BLOCK_SIZE), temp(SORT_THRESHOLD);
  // The reference sizes the stack QUICKSORT_BLOCK_SIZE/SORT_THRESHOLD (line 280);
  // every pushed run is longer than SORT_THRESHOLD and the runs on the stack are
  // disjoint, so that bound holds.
  workstack_record workstack[QUICKSORT_BLOCK_SIZE / SORT_THRESHOLD + 1];
  int wp = 0;
  const uint32_t d_offset = block.start;
  uint32_t end = block.end - d_offset;
  workstack[0] = workstack_record{0, end, 1};
  const T* src = block.direction == 1 ? d : dn;
  for (uint32_t i = 0; i < end; ++i) mys[i] = src[i + d_offset];
  T* out = d + d_offset;
  uint32_t lt[WG + 1], gt[WG + 1];
  while (wp >= 0) {
    workstack_record wr = workstack[wp--];
    uint32_t start = wr.start;
    end = wr.end;
    uint32_t direction = wr.direction;
    T* s = direction == 1 ? mys.data() : mysn.data();
    T* sn = direction == 1 ? mysn.data() : mys.data();
    T pivot = s[start];
    if (start < end) pivot = median(pivot, s[(start + end) >> 1], s[end - 1]);
    for (uint32_t l = 0; l < WG; ++l) {
      uint32_t ltp = 0, gtp = 0;
      for (uint32_t i = start + l; i < end; i += WG) {
        T tmp = s[i];
        if (tmp < pivot) ++ltp;
        if (tmp > pivot) ++gtp;
      }
      lt[l] = ltp;
      gt[l] = gtp;
    }
    uint32_t ltsum = exclusive_scan(lt, WG);
    uint32_t gtsum = exclusive_scan(gt, WG);
    lt[WG] = ltsum;
    gt[WG] = gtsum;
    // Greater keys of work-item l land in [end - gt[l+1], end - gt[l]) (lines 386-398).
    for (uint32_t l = 0; l < WG; ++l) {
      uint32_t lfrom = start + lt[l], gfrom = end - gt[l + 1];
      for (uint32_t i = start + l; i < end; i += WG) {
        T tmp = s[i];
        if (tmp < pivot) sn[lfrom++] = tmp;
        if (tmp > pivot) sn[gfrom++] = tmp;
      }
    }
    for (uint32_t i = start + ltsum; i < end - gtsum; ++i) out[i] = pivot;  // lines 402-404
    if (ltsum <= SORT_THRESHOLD) {
      sort_threshold(sn, out, start, start + ltsum, temp.data());
    } else {
      workstack[++wp] = workstack_record{start, start + ltsum, direction ^ 1u};
    }
    if (gtsum <= SORT_THRESHOLD) {
      sort_threshold(sn, out, end - gtsum, end, temp.data());
    } else {
      workstack[++wp] = workstack_record{end - gtsum, end, direction ^ 1u};
    }
  }
}

struct oracle_stats_t {
  uint64_t levels;        // gqsort launches
  uint64_t active_keys;   // sum over levels of the keys in work records
  uint64_t blocks;        // gqsort work-groups launched, all levels
  uint64_t done_records;  // lqsort work-groups
  uint64_t maxseq;
};

// The host level loop of GPUQSort<T> (QuicksortMain.cpp:835-906).
template <class T>
int gpuqsort(T* d, T* dn, size_t size, int threads, oracle_stats_t* st) {
  if (size == 0) return 0;
  if (size >= (1ull << 32)) return -1;  // record fields are 32-bit (Quicksort.h:147-148)
  if (threads < 1) threads = 1;
  const size_t MAXSEQ = optp(size, 0.00009516, 203);
  T startpivot = median(d[0], d[size / 2], d[size - 1]);
  std::vector<work_record<T>> work, done, news;
  std::vector<parent_record> parent_records;
  std::vector<block_record<T>> blocks;
  work.push_back(work_record<T>{0, (uint32_t)size, startpivot, 1});
  oracle_stats_t s{};
  s.maxseq = MAXSEQ;
  while (!work.empty()) {
    size_t blocksize = 0;
    for (auto& w : work) blocksize += std::max<size_t>((w.end - w.start) / MAXSEQ, 1);
    for (auto& w : work) {
      s.active_keys += w.end - w.start;
      uint32_t blockcount = (uint32_t)((w.end - w.start + blocksize - 1) / blocksize);
      parent_records.push_back(parent_record{w.start, w.end, w.start, w.end, blockcount - 1});
      uint32_t prnt = (uint32_t)parent_records.size() - 1;
      for (uint32_t i = 0; i + 1 < blockcount; ++i) {
        uint32_t bstart = w.start + (uint32_t)(blocksize * i);
        blocks.push_back(block_record<T>{bstart, bstart + (uint32_t)blocksize, w.pivot, w.direction, prnt});
      }
      blocks.push_back(block_record<T>{w.start + (uint32_t)(blocksize * (blockcount - 1)), w.end, w.pivot,
                                       w.direction, prnt});
    }
    news.assign(blocks.size() * 2, work_record<T>{});
    s.levels += 1;
    s.blocks += blocks.size();
    const long long nb = (long long)blocks.size();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) if (threads > 1)
    for (long long b = 0; b < nb; ++b) gqsort_block(d, dn, blocks[b], parent_records.data(), news.data(), (size_t)b);
    work.clear();
    parent_records.clear();
    blocks.clear();
    for (auto& r : news) {
      if (r.direction == EMPTY_RECORD) continue;
      if (r.end - r.start <= QUICKSORT_BLOCK_SIZE) {
        if (r.end - r.start > 0) done.push_back(r);
      } else {
        work.push_back(r);
      }
    }
  }
  s.done_records = done.size();
  const long long nd = (long long)done.size();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16) if (threads > 1)
  for (long long r = 0; r < nd; ++r) lqsort_record(d, dn, done[r]);
  if (st) *st = s;
  return 0;
}

// The reference's CPU quicksort<T> (QuicksortMain.cpp:213-259): Lomuto
// partition around data[left] moved to the right end, std::sort for runs of
// at most 33 keys. Recursion is replaced by an explicit stack with the same
// visiting order, so adversarial inputs cannot overflow the host stack.
template <class T>
T* ref_partition(T* left, T* right, T pivot) {
  T temp = *right;
  *right = pivot;
  *left = temp;
  T* store = left;
  for (T* p = left; p != right; ++p) {
    if (*p < pivot) {
      temp = *store;
      *store = *p;
      *p = temp;
      ++store;
    }
  }
  temp = *store;
  *store = pivot;
  *right = temp;
  return store;
}

template <class T>
void ref_cpu_quicksort(T* data, long long left, long long right) {
  std::vector<std::pair<long long, long long>> stack;
  stack.emplace_back(left, right);
  while (!stack.empty()) {
    auto [l, r] = stack.back();
    stack.pop_back();
    T* store = ref_partition(data + l, data + r, data[l]);
    long long nright = store - data;
    long long nleft = nright + 1;
    // The recursive original visits the left part first; push it last.
    if (nleft < r) {
      if (r - nleft > 32) stack.emplace_back(nleft, r);
      else std::sort(data + nleft, data + r + 1);
    }
    if (l < nright) {
      if (nright - l > 32) stack.emplace_back(l, nright);
      else std::sort(data + l, data + nright + 1);
    }
  }
}

}  // namespace

extern "C" {

typedef oracle_stats_t oracle_stats;

int oracle_gpuqsort_u32(uint32_t* d, uint32_t* dn, size_t n, int threads, oracle_stats* st) {
  return gpuqsort(d, dn, n, threads, st);
}
int oracle_gpuqsort_f32(float* d, float* dn, size_t n, int threads, oracle_stats* st) {
  return gpuqsort(d, dn, n, threads, st);
}
int oracle_gpuqsort_f64(double* d, double* dn, size_t n, int threads, oracle_stats* st) {
  return gpuqsort(d, dn, n, threads, st);
}

void oracle_std_sort_u32(uint32_t* d, size_t n) { std::sort(d, d + n); }
void oracle_std_sort_f32(float* d, size_t n) { std::sort(d, d + n); }
void oracle_std_sort_f64(double* d, size_t n) { std::sort(d, d + n); }

void oracle_parallel_sort_u32(uint32_t* d, size_t n, int threads) {
  omp_set_num_threads(threads < 1 ? 1 : threads);
  __gnu_parallel::sort(d, d + n);
}
void oracle_parallel_sort_f32(float* d, size_t n, int threads) {
  omp_set_num_threads(threads < 1 ? 1 : threads);
  __gnu_parallel::sort(d, d + n);
}
void oracle_parallel_sort_f64(double* d, size_t n, int threads) {
  omp_set_num_threads(threads < 1 ? 1 : threads);
  __gnu_parallel::sort(d, d + n);
}

void oracle_cpu_quicksort_u32(uint32_t* d, size_t n) { if (n > 1) ref_cpu_quicksort(d, 0, (long long)n - 1); }
void oracle_cpu_quicksort_f32(float* d, size_t n) { if (n > 1) ref_cpu_quicksort(d, 0, (long long)n - 1); }
void oracle_cpu_quicksort_f64(double* d, size_t n) { if (n > 1) ref_cpu_quicksort(d, 0, (long long)n - 1); }

// Segmented form: every segment [off[i], off[i+1]) is sorted independently
// with the GPUQSort<T> restatement.
int oracle_gpuqsort_segments_u32(uint32_t* d, uint32_t* dn, const uint64_t* off, size_t nseg, int threads) {
  int rc = 0;
#pragma omp parallel for num_threads(threads < 1 ? 1 : threads) schedule(dynamic, 1) reduction(| : rc)
  for (long long s = 0; s < (long long)nseg; ++s)
    rc |= gpuqsort(d + off[s], dn + off[s], (size_t)(off[s + 1] - off[s]), 1, nullptr);
  return rc;
}

}  // extern "C"
