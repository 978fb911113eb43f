// Mixed-precision (fp32 pair arithmetic) form of the per-leaf kernels; see kernels.cuh.
#include "kernels.cuh"
