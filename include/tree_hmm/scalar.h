// tree_hmm::Scalar, the library's compile-time floating-point type: double by
// default, float with TREE_HMM_USE_FLOAT (the same switch and include guard as
// the reference's include/tree_hmm/scalar.h:1-16, so either header can serve).
#ifndef TREE_HMM_SCALAR_H_
#define TREE_HMM_SCALAR_H_

namespace tree_hmm {

#ifdef TREE_HMM_USE_FLOAT
using Scalar = float;
inline constexpr const char *kPrecisionName = "FP32";
#else
using Scalar = double;
inline constexpr const char *kPrecisionName = "FP64";
#endif

} // namespace tree_hmm

#endif // TREE_HMM_SCALAR_H_
