// Kernels of the ur5 robot (generated FK and check schedule in robots/ur5.cuh).
#include "robots/ur5.cuh"
#include "vg_robot.cuh"

// register-rich same-edge schedule: the autotuner's pick on 16,384 edges in the
// 60-primitive + pointcloud scene
VG_DEFINE_ROBOT(Ur5, ops_ur5, 2)
