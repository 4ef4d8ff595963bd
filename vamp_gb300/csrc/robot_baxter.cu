// Kernels of the baxter robot (generated FK and check schedule in robots/baxter.cuh).
#include "robots/baxter.cuh"
#include "vg_robot.cuh"

// same-edge schedule: the autotuner's pick on 16,384 edges in the 60-primitive +
// pointcloud scene
VG_DEFINE_ROBOT(Baxter, ops_baxter, 1)
