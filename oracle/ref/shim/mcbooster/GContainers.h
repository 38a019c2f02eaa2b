// Project-written stand-ins for MCBooster's container names: Thrust vectors of the build's device system,
// sets of pointers to them, and a strided view over an iterator range.
#pragma once
#include <mcbooster/GTypes.h>
#include <mcbooster/Vector4R.h>
#include <thrust/device_vector.h>
#include <thrust/functional.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/permutation_iterator.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/reduce.h>
#include <thrust/transform.h>
#include <thrust/transform_reduce.h>
#include <vector>

namespace mcbooster {
template <typename T>
using mc_device_vector = thrust::device_vector<T>;
template <typename T>
using mc_host_vector = thrust::host_vector<T>;
typedef mc_device_vector<GReal_t> RealVector_d;
typedef mc_host_vector<GReal_t> RealVector_h;
typedef mc_device_vector<GBool_t> BoolVector_d;
typedef mc_host_vector<GBool_t> BoolVector_h;
typedef mc_device_vector<Vector4R> Particles_d;
typedef mc_host_vector<Vector4R> Particles_h;
typedef std::vector<Particles_d *> ParticlesSet_d;
typedef std::vector<Particles_h *> ParticlesSet_h;
typedef std::vector<RealVector_d *> VariableSet_d;
typedef std::vector<RealVector_h *> VariableSet_h;

// every stride-th element of [first, last)
template <typename Iterator>
class strided_range {
  public:
    typedef typename thrust::iterator_difference<Iterator>::type difference_type;
    struct stride_functor {
        difference_type stride;
        explicit stride_functor(difference_type s) : stride(s) {}
        __host__ __device__ difference_type operator()(const difference_type &i) const { return stride * i; }
    };
    typedef thrust::transform_iterator<stride_functor, thrust::counting_iterator<difference_type>> IndexIterator;
    typedef thrust::permutation_iterator<Iterator, IndexIterator> iterator;

    strided_range(Iterator first, Iterator last, difference_type stride)
        : first_(first), last_(last), stride_(stride) {}
    iterator begin() const {
        return iterator(first_, IndexIterator(thrust::counting_iterator<difference_type>(0), stride_functor(stride_)));
    }
    iterator end() const { return begin() + ((last_ - first_) + (stride_ - 1)) / stride_; }

  private:
    Iterator first_, last_;
    difference_type stride_;
};
} // namespace mcbooster
