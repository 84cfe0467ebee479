/* Pre-included when the reference Lanczos solver is compiled for the CPU with
 * thrust's host (CPP) device system: the solver names thrust::cuda::par
 * (include/lanczos/utils/device_container.h:9-17), which here becomes the
 * sequential host policy.  TEST INFRASTRUCTURE ONLY. */
#pragma once
#include <thrust/execution_policy.h>
namespace thrust {
namespace cuda {
static const auto &par = thrust::cpp::par;
}
} // namespace thrust
