// cuda_copy<T, predicate> (the reference's src/reduction/cuda_copy.hpp)
// re-implemented with Thrust for the build of the reference's GPU miner used
// as a second oracle: copy_if keeps, in order, the elements whose INDEX
// satisfies the predicate and returns their count.  TEST INFRASTRUCTURE
// ONLY (oracle/gspan_cuda.mk puts it in place of the library's MGPU version,
// whose scan relies on implicit warp lock-step).
#include <thrust/copy.h>
#include <thrust/execution_policy.h>
#include <thrust/iterator/counting_iterator.h>

template<class T, class predicate>
cuda_copy<T, predicate>::cuda_copy()
{
  remap_array = 0;
  remap_array_length = 0;
  logger = Logger::get_logger("CC");
}

template<class T, class predicate>
cuda_copy<T, predicate>::~cuda_copy()
{
}

template<class T, class predicate>
void cuda_copy<T, predicate>::remap_input_array(uint *, int, reduce_type_t, predicate)
{
}

template<class T, class predicate>
int cuda_copy<T, predicate>::copy_if(T *array_begin, int length, T *to_array_begin, predicate p)
{
  if(length <= 0) return 0;
  T *end = thrust::copy_if(thrust::device, array_begin, array_begin + length, thrust::counting_iterator<int>(0),
                           to_array_begin, p);
  cudaDeviceSynchronize();
  return (int)(end - to_array_begin);
}
