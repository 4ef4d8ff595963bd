// Kernels of the ur5 robot (generated FK and check schedule in robots/ur5.cuh).
#include "robots/ur5.cuh"
#include "vg_robot.cuh"

VG_DEFINE_ROBOT(Ur5, ops_ur5)
