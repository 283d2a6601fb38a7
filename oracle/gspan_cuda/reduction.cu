// The reference's reduction library (src/reduction: cuda_segmented_scan,
// cuda_segmented_reduction) re-implemented with Thrust, for the build of the
// reference's GPU miner (gspan_cuda_no_sort) used as a second oracle.
//
// TEST INFRASTRUCTURE ONLY: compiled by oracle/gspan_cuda.mk into
// oracle/_ref/ with the reference's own sources; the product never links it.
//
// Why: the library's kernels (MGPU-era segmented scans, scancommon.cu,
// segscanpacked.cu, segreducepacked2.cu) rely on the implicit lock-step of a
// warp -- volatile shared-memory scans without warp barriers, __ballot -- which
// GPUs since Volta do not provide.  The class interfaces stay the reference's
// (src/reduction/cuda_segmented_op.hpp, cuda_segmented_reduction.hpp,
// cuda_segmented_scan.hpp); only the bodies are new:
//   * packed layout: bit 31 of an element starts a segment (element 0 always
//     does), bits 0-30 are its value; results are unpacked sums;
//   * scan = inclusive or exclusive scan by segment key (the running count
//     of segment starts);
//   * reduce = that scan read at the last element of every segment, the
//     segments given as runs of equal sizes (cuda_segmented_reduction.cpp:
//     98-134).
#include <cuda_segmented_op.hpp>
#include <cuda_segmented_reduction.hpp>
#include <cuda_segmented_scan.hpp>

#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/scan.h>
#include <thrust/transform.h>

namespace {

struct head_of {
  const uint *in;
  __host__ __device__ uint operator()(int i) const { return (i == 0 || (in[i] >> 31)) ? 1u : 0u; }
};

struct value_of {
  __host__ __device__ uint operator()(uint x) const { return x & 0x7fffffffu; }
};

void packed_scan(const uint *d_in, uint *d_out, int count, bool inclusive)
{
  if(count <= 0) return;
  thrust::device_vector<uint> key(count), val(count);
  thrust::transform(thrust::device, thrust::counting_iterator<int>(0), thrust::counting_iterator<int>(count),
                    key.begin(), head_of{ d_in });
  thrust::inclusive_scan(thrust::device, key.begin(), key.end(), key.begin());
  thrust::transform(thrust::device, thrust::device_pointer_cast(d_in), thrust::device_pointer_cast(d_in) + count,
                    val.begin(), value_of());
  thrust::device_ptr<uint> out = thrust::device_pointer_cast(d_out);
  if(inclusive) thrust::inclusive_scan_by_key(thrust::device, key.begin(), key.end(), val.begin(), out);
  else thrust::exclusive_scan_by_key(thrust::device, key.begin(), key.end(), val.begin(), out, 0u);
  cudaDeviceSynchronize();
}

}  // namespace

cuda_segmented_op::cuda_segmented_op()
    : logger(Logger::get_logger("CUDA_PP")), blockScanMem(0), blockScanMem_size(0), headFlagsMem(0),
      headFlagsMem_size(0), ranges(0), ranges_size(0), d_reduce_result(0), d_reduce_result_size(0),
      d_segmented_count(0), d_segmented_count_size(0), d_segmented_sizes(0), d_segmented_sizes_size(0)
{
}

cuda_segmented_op::~cuda_segmented_op() {}

cuda_segmented_scan::cuda_segmented_scan() {}
cuda_segmented_scan::~cuda_segmented_scan() {}

void cuda_segmented_scan::scan(uint *d_in, uint *d_out, int count, reduce_type_t inclusive)
{
  packed_scan(d_in, d_out, count, inclusive == INCLUSIVE);
}

void cuda_segmented_scan::global_scan(uint *d_in, uint *d_out, int count, reduce_type_t inclusive)
{
  if(count <= 0) return;
  thrust::device_ptr<uint> in = thrust::device_pointer_cast(d_in), out = thrust::device_pointer_cast(d_out);
  if(inclusive == INCLUSIVE) thrust::inclusive_scan(thrust::device, in, in + count, out);
  else thrust::exclusive_scan(thrust::device, in, in + count, out, 0u);
  cudaDeviceSynchronize();
}

cuda_segmented_reduction::cuda_segmented_reduction() {}
cuda_segmented_reduction::~cuda_segmented_reduction() {}

void cuda_segmented_reduction::reduce(uint *d_array_packed, int count, std::vector<uint> segment_count,
                                      std::vector<uint> segment_sizes, std::vector<uint> &results,
                                      reduce_type_t inclusive)
{
  results.clear();
  if(count <= 0) return;
  thrust::device_vector<uint> scanned(count);
  packed_scan(d_array_packed, thrust::raw_pointer_cast(scanned.data()), count, inclusive == INCLUSIVE);
  std::vector<uint> host(count);
  thrust::copy(scanned.begin(), scanned.end(), host.begin());
  long long at = 0;
  for(size_t g = 0; g < segment_sizes.size() && g < segment_count.size(); g++)
    for(uint c = 0; c < segment_count[g]; c++) {
      at += segment_sizes[g];
      results.push_back(at - 1 < count ? host[at - 1] : 0u);
    }
}

void cuda_segmented_reduction::reduce_inclusive(uint *d_array_packed, int count, std::vector<uint> segment_count,
                                                std::vector<uint> segment_sizes, std::vector<uint> &results)
{
  reduce(d_array_packed, count, segment_count, segment_sizes, results, INCLUSIVE);
}

void cuda_segmented_reduction::reduce_exclusive(uint *d_array_packed, int count, std::vector<uint> segment_count,
                                                std::vector<uint> segment_sizes, std::vector<uint> &results)
{
  reduce(d_array_packed, count, segment_count, segment_sizes, results, EXCLUSIVE);
}
