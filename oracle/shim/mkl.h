// Stand-in for <mkl.h>.  TEST INFRASTRUCTURE ONLY: the reference's CSR builder
// (cpp/core/csr_local.hpp:13) includes it for the sparse BLAS declarations only.
#pragma once
#include "mkl_spblas.h"
