// Plan-update, rho and layout-conversion kernels instantiated for MP = 8
// (one translation unit per padded support size, compiled in parallel).
#include "plan_kernel.cuh"
namespace d2g {
D2G_INSTANTIATE_MP(8)
}
