// Kernels of the fetch robot (generated FK and check schedule in robots/fetch.cuh).
#include "robots/fetch.cuh"
#include "vg_robot.cuh"

// register-rich same-edge schedule: the autotuner's pick on 16,384 edges in the
// 60-primitive + pointcloud scene
VG_DEFINE_ROBOT(Fetch, ops_fetch, 2)
