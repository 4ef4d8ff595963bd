// Kernels of the panda robot (generated FK and check schedule in robots/panda.cuh).
#include "robots/panda.cuh"
#include "vg_robot.cuh"

VG_DEFINE_ROBOT(Panda, ops_panda)
