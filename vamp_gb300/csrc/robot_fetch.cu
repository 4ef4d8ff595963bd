// Kernels of the fetch robot (generated FK and check schedule in robots/fetch.cuh).
#include "robots/fetch.cuh"
#include "vg_robot.cuh"

VG_DEFINE_ROBOT(Fetch, ops_fetch)
