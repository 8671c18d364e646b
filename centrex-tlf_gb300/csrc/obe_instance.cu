// obe_instance.cu -- one kernel shape per compilation: the build compiles this file once per
// (threads per trajectory, elements per thread) pair, -DOBE_TPT=.. -DOBE_EPT=.., which
// instantiates the integrator in both forms (and, with -DOBE_RHS, the RHS kernel of that width;
// up to 256 threads per trajectory also the adjoint kernel).
#define OBE_INSTANCE_TU
#include "obe_kernels.cuh"
#include "obe_adjoint.cuh"

#if !defined(OBE_TPT) || !defined(OBE_EPT)
#error "obe_instance.cu is compiled once per kernel shape: define OBE_TPT and OBE_EPT"
#endif

namespace obe {
template cudaError_t launch_integrate_shape<OBE_TPT, OBE_EPT, false>(const DevPlan&, const CallArgs&, int, int, size_t, size_t,
                                                                     int, cudaStream_t);
template cudaError_t launch_integrate_shape<OBE_TPT, OBE_EPT, true>(const DevPlan&, const CallArgs&, int, int, size_t, size_t,
                                                                    int, cudaStream_t);
#ifdef OBE_RHS
template cudaError_t launch_rhs_shape<OBE_TPT, false>(const DevPlan&, long long, const double*, const double*, int, const int*,
                                                      const double*, double*, int, int, size_t, size_t, int, unsigned char*,
                                                      size_t, double*);
template cudaError_t launch_rhs_shape<OBE_TPT, true>(const DevPlan&, long long, const double*, const double*, int, const int*,
                                                     const double*, double*, int, int, size_t, size_t, int, unsigned char*,
                                                     size_t, double*);
#endif
#if OBE_TPT <= 256
template cudaError_t launch_adjoint_shape<OBE_TPT, OBE_EPT, false>(const DevPlan&, const CallArgs&, const AdjArgs&, int, int,
                                                                   size_t, size_t, int, cudaStream_t);
template cudaError_t launch_adjoint_shape<OBE_TPT, OBE_EPT, true>(const DevPlan&, const CallArgs&, const AdjArgs&, int, int,
                                                                  size_t, size_t, int, cudaStream_t);
#endif
}  // namespace obe
