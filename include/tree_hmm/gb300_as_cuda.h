// Source-level drop-in for code written against the reference's
// tree_hmm::cuda (include/tree_hmm/cuda.h): makes tree_hmm::cuda name the GB300
// implementation. Include instead of the reference's tree_hmm/cuda.h.
#ifndef TREE_HMM_GB300_AS_CUDA_H_
#define TREE_HMM_GB300_AS_CUDA_H_

#include "tree_hmm/gb300.h"

namespace tree_hmm {
namespace cuda = gb300;
} // namespace tree_hmm

#endif // TREE_HMM_GB300_AS_CUDA_H_
