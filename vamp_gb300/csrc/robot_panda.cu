// Kernels of the panda robot (generated FK and check schedule in robots/panda.cuh).
#include "robots/panda.cuh"
#include "vg_robot.cuh"

// register-rich same-edge schedule: the autotuner's pick on the 65,536-edge workload, and
// the fastest on the batched roadmap's PRM* edges and on shorter edges
VG_DEFINE_ROBOT(Panda, ops_panda, 2)
