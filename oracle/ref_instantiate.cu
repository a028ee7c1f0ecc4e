// Build recipe input for the reference's own kernels (oracle/_ref/, test
// infrastructure only).  Compiles the unmodified reference sources, taken from
// the reference checkout through the include path, into a device-only cubin
// for sm_103a.  The reference's packers are templates, so they are explicitly
// instantiated here for float input, as its drivers use them
// (bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:107,230,353,476;
// bmv_eval/test_bin_bin_bin.cu:257-280).  Nothing of the reference is copied.
#include "bsrbmv.cu"

template __global__ void ToBit4Col<float>(const float*, uchar*, const int);
template __global__ void ToBit8Col<float>(const float*, uchar*, const int);
template __global__ void ToBit16Col<float>(const float*, ushort*, const int);
template __global__ void ToBit32Col<float>(const float*, unsigned*, const int, const int);
template __global__ void ToBit4Row<float>(const float*, uchar*, const int);
template __global__ void ToBit8Row<float>(const float*, uchar*, const int);
template __global__ void ToBit16Row<float>(const float*, ushort*, const int);
template __global__ void ToBit32Row<float>(const float*, unsigned*, const int);
