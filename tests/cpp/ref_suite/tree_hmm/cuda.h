// Test-only forwarding header: lets the reference's own accelerator suite
// (tests/cuda_test.cc, which includes "tree_hmm/cuda.h") compile against this
// library's drop-in, tree_hmm::gb300 exposed as tree_hmm::cuda. Nothing of
// the reference's CUDA backend is involved.
#ifndef THMM_TESTS_REF_SUITE_TREE_HMM_CUDA_H_
#define THMM_TESTS_REF_SUITE_TREE_HMM_CUDA_H_

#include "tree_hmm/gb300_as_cuda.h"

#endif // THMM_TESTS_REF_SUITE_TREE_HMM_CUDA_H_
