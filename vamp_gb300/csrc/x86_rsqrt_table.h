// The x86 RSQRTPS results on [1, 4) (see vg_check.cuh, rsqrt_x86), generated by
// oracle/ref/gen_rsqrt_table.c on an x86-64 CPU and checked there against every positive float.
#pragma once
#include <cstdint>

namespace vg
{
    static const uint32_t kX86RsqrtTable[2048] = {
#include "x86_rsqrt_table.inc"
    };
}
