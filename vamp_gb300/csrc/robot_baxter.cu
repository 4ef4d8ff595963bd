// Kernels of the baxter robot (generated FK and check schedule in robots/baxter.cuh).
#include "robots/baxter.cuh"
#include "vg_robot.cuh"

VG_DEFINE_ROBOT(Baxter, ops_baxter)
