// Generated by vamp_gb300/robotgen/codegen.py from vamp_gb300/robots/panda.json. Do not edit.
//
// FP32 forward kinematics and the fkcc check schedule of the panda robot, one configuration
// per thread.  Schedule order follows the reference's generated Robot::fkcc
// (src/impl/vamp/robots/panda.hh): environment checks link by link, each a coarse link sphere
// gating that link's fine spheres, then self-collision link pairs, a coarse pair gating the
// cross product of the two links' fine spheres.  Schedule form: straight-line.
#pragma once

#include "../vg_check.cuh"

namespace vg::robots
{
struct Panda
{
    static constexpr const char *kName = "panda";
    static constexpr int kDim = 7;
    static constexpr int kFine = 59;
    static constexpr int kSlots = 70;
    static constexpr int kFrames = 8;
    static constexpr int kResolution = 32;
    static constexpr float kMinRadius = 0.012000000104308128f;
    static constexpr float kMaxRadius = 0.07999999821186066f;
    static constexpr float kScaleM[7] = {5.934199810028076f, 3.6651999950408936f, 5.934199810028076f, 3.2288999557495117f, 5.934199810028076f, 3.909600019454956f, 5.934199810028076f};
    static constexpr float kScaleA[7] = {-2.967099905014038f, -1.8325999975204468f, -2.967099905014038f, -3.1415998935699463f, -2.967099905014038f, -0.08730000257492065f, -2.967099905014038f};

    // Every sphere slot: fine spheres 0..kFine-1, then the coarse sphere of each checked link.
    static __device__ __forceinline__ void spheres(const float *q, float *out)
    {
        float F0_s, F0_c; vg_sincos_ref(q[0], &F0_s, &F0_c);
        const float F0_r00 = F0_c;
        const float F0_r01 = (-F0_s);
        const float F0_r10 = F0_s;
        const float F0_r11 = F0_c;
        float F1_s, F1_c; vg_sincos_ref(q[1], &F1_s, &F1_c);
        const float F1_r00 = __fmul_rn(F0_r00, F1_c);
        const float F1_r01 = __fmul_rn((-F0_r00), F1_s);
        const float F1_r02 = F0_r01;
        const float F1_r10 = __fmul_rn(F0_r10, F1_c);
        const float F1_r11 = __fmul_rn((-F0_r10), F1_s);
        const float F1_r12 = F0_r11;
        const float F1_r20 = (-F1_s);
        const float F1_r21 = (-F1_c);
        const float _v4 = __fmul_rn(-0.3160000145435333f, F1_r01);
        const float _v5 = __fmul_rn(-0.3160000145435333f, F1_r11);
        const float _v6 = __fmaf_rn(-0.3160000145435333f, F1_r21, 0.3330000042915344f);
        float F2_s, F2_c; vg_sincos_ref(q[2], &F2_s, &F2_c);
        const float _v7 = __fmul_rn(F1_r00, F2_c);
        const float F2_r00 = __fmaf_rn(F1_r02, F2_s, _v7);
        const float _v9 = __fmul_rn((-F1_r00), F2_s);
        const float F2_r01 = __fmaf_rn(F1_r02, F2_c, _v9);
        const float F2_r02 = (-F1_r01);
        const float _v11 = __fmul_rn(F1_r10, F2_c);
        const float F2_r10 = __fmaf_rn(F1_r12, F2_s, _v11);
        const float _v13 = __fmul_rn((-F1_r10), F2_s);
        const float F2_r11 = __fmaf_rn(F1_r12, F2_c, _v13);
        const float F2_r12 = (-F1_r11);
        const float F2_r20 = __fmul_rn(F1_r20, F2_c);
        const float F2_r21 = __fmul_rn((-F1_r20), F2_s);
        const float F2_r22 = (-F1_r21);
        const float F2_t0 = _v4;
        const float F2_t1 = _v5;
        const float F2_t2 = _v6;
        const float _v17 = __fmaf_rn(0.08250000327825546f, F2_r00, F2_t0);
        const float _v18 = __fmaf_rn(0.08250000327825546f, F2_r10, F2_t1);
        const float _v19 = __fmaf_rn(0.08250000327825546f, F2_r20, F2_t2);
        float F3_s, F3_c; vg_sincos_ref(q[3], &F3_s, &F3_c);
        const float _v20 = __fmul_rn(F2_r00, F3_c);
        const float F3_r00 = __fmaf_rn(F2_r02, F3_s, _v20);
        const float _v22 = __fmul_rn((-F2_r00), F3_s);
        const float F3_r01 = __fmaf_rn(F2_r02, F3_c, _v22);
        const float F3_r02 = (-F2_r01);
        const float _v24 = __fmul_rn(F2_r10, F3_c);
        const float F3_r10 = __fmaf_rn(F2_r12, F3_s, _v24);
        const float _v26 = __fmul_rn((-F2_r10), F3_s);
        const float F3_r11 = __fmaf_rn(F2_r12, F3_c, _v26);
        const float F3_r12 = (-F2_r11);
        const float _v28 = __fmul_rn(F2_r20, F3_c);
        const float F3_r20 = __fmaf_rn(F2_r22, F3_s, _v28);
        const float _v30 = __fmul_rn((-F2_r20), F3_s);
        const float F3_r21 = __fmaf_rn(F2_r22, F3_c, _v30);
        const float F3_r22 = (-F2_r21);
        const float F3_t0 = _v17;
        const float F3_t1 = _v18;
        const float F3_t2 = _v19;
        const float _v32 = __fmaf_rn(-0.08250000327825546f, F3_r00, F3_t0);
        const float _v33 = __fmaf_rn(0.3840000033378601f, F3_r01, _v32);
        const float _v34 = __fmaf_rn(-0.08250000327825546f, F3_r10, F3_t1);
        const float _v35 = __fmaf_rn(0.3840000033378601f, F3_r11, _v34);
        const float _v36 = __fmaf_rn(-0.08250000327825546f, F3_r20, F3_t2);
        const float _v37 = __fmaf_rn(0.3840000033378601f, F3_r21, _v36);
        float F4_s, F4_c; vg_sincos_ref(q[4], &F4_s, &F4_c);
        const float _v38 = __fmul_rn(F3_r00, F4_c);
        const float F4_r00 = __fmaf_rn((-F3_r02), F4_s, _v38);
        const float _v40 = __fmul_rn((-F3_r00), F4_s);
        const float F4_r01 = __fmaf_rn((-F3_r02), F4_c, _v40);
        const float F4_r02 = F3_r01;
        const float _v42 = __fmul_rn(F3_r10, F4_c);
        const float F4_r10 = __fmaf_rn((-F3_r12), F4_s, _v42);
        const float _v44 = __fmul_rn((-F3_r10), F4_s);
        const float F4_r11 = __fmaf_rn((-F3_r12), F4_c, _v44);
        const float F4_r12 = F3_r11;
        const float _v46 = __fmul_rn(F3_r20, F4_c);
        const float F4_r20 = __fmaf_rn((-F3_r22), F4_s, _v46);
        const float _v48 = __fmul_rn((-F3_r20), F4_s);
        const float F4_r21 = __fmaf_rn((-F3_r22), F4_c, _v48);
        const float F4_r22 = F3_r21;
        const float F4_t0 = _v33;
        const float F4_t1 = _v35;
        const float F4_t2 = _v37;
        float F5_s, F5_c; vg_sincos_ref(q[5], &F5_s, &F5_c);
        const float _v50 = __fmul_rn(F4_r00, F5_c);
        const float F5_r00 = __fmaf_rn(F4_r02, F5_s, _v50);
        const float _v52 = __fmul_rn((-F4_r00), F5_s);
        const float F5_r01 = __fmaf_rn(F4_r02, F5_c, _v52);
        const float F5_r02 = (-F4_r01);
        const float _v54 = __fmul_rn(F4_r10, F5_c);
        const float F5_r10 = __fmaf_rn(F4_r12, F5_s, _v54);
        const float _v56 = __fmul_rn((-F4_r10), F5_s);
        const float F5_r11 = __fmaf_rn(F4_r12, F5_c, _v56);
        const float F5_r12 = (-F4_r11);
        const float _v58 = __fmul_rn(F4_r20, F5_c);
        const float F5_r20 = __fmaf_rn(F4_r22, F5_s, _v58);
        const float _v60 = __fmul_rn((-F4_r20), F5_s);
        const float F5_r21 = __fmaf_rn(F4_r22, F5_c, _v60);
        const float F5_r22 = (-F4_r21);
        const float F5_t0 = F4_t0;
        const float F5_t1 = F4_t1;
        const float F5_t2 = F4_t2;
        const float _v62 = __fmaf_rn(0.08799999952316284f, F5_r00, F5_t0);
        const float _v63 = __fmaf_rn(0.08799999952316284f, F5_r10, F5_t1);
        const float _v64 = __fmaf_rn(0.08799999952316284f, F5_r20, F5_t2);
        float F6_s, F6_c; vg_sincos_ref(q[6], &F6_s, &F6_c);
        const float _v65 = __fmul_rn(F5_r00, F6_c);
        const float F6_r00 = __fmaf_rn(F5_r02, F6_s, _v65);
        const float _v67 = __fmul_rn((-F5_r00), F6_s);
        const float F6_r01 = __fmaf_rn(F5_r02, F6_c, _v67);
        const float F6_r02 = (-F5_r01);
        const float _v69 = __fmul_rn(F5_r10, F6_c);
        const float F6_r10 = __fmaf_rn(F5_r12, F6_s, _v69);
        const float _v71 = __fmul_rn((-F5_r10), F6_s);
        const float F6_r11 = __fmaf_rn(F5_r12, F6_c, _v71);
        const float F6_r12 = (-F5_r11);
        const float _v73 = __fmul_rn(F5_r20, F6_c);
        const float F6_r20 = __fmaf_rn(F5_r22, F6_s, _v73);
        const float _v75 = __fmul_rn((-F5_r20), F6_s);
        const float F6_r21 = __fmaf_rn(F5_r22, F6_c, _v75);
        const float F6_r22 = (-F5_r21);
        const float F6_t0 = _v62;
        const float F6_t1 = _v63;
        const float F6_t2 = _v64;
        const float _v77 = __fmaf_rn(1.0f, 0.0f, 0.0f);
        const float _v78 = __fmaf_rn(0.0f, 0.0f, _v77);
        const float s0_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v78);
        const float _v80 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v81 = __fmaf_rn(1.0f, 0.0f, _v80);
        const float s0_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v81);
        const float _v83 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v84 = __fmaf_rn(0.0f, 0.0f, _v83);
        const float s0_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v84);
        out[0] = s0_x; out[1] = s0_y; out[2] = s0_z; out[3] = 0.07999999821186066f;
        const float _v86 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v87 = __fmaf_rn(F0_r01, -0.07999999821186066f, _v86);
        const float s1_x = __fmaf_rn(0.0f, 0.0f, _v87);
        const float _v89 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v90 = __fmaf_rn(F0_r11, -0.07999999821186066f, _v89);
        const float s1_y = __fmaf_rn(0.0f, 0.0f, _v90);
        const float _v92 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v93 = __fmaf_rn(0.0f, -0.07999999821186066f, _v92);
        const float s1_z = __fmaf_rn(1.0f, 0.0f, _v93);
        out[4] = s1_x; out[5] = s1_y; out[6] = s1_z; out[7] = 0.05999999865889549f;
        const float _v95 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v96 = __fmaf_rn(F0_r01, -0.029999999329447746f, _v95);
        const float s2_x = __fmaf_rn(0.0f, 0.0f, _v96);
        const float _v98 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v99 = __fmaf_rn(F0_r11, -0.029999999329447746f, _v98);
        const float s2_y = __fmaf_rn(0.0f, 0.0f, _v99);
        const float _v101 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v102 = __fmaf_rn(0.0f, -0.029999999329447746f, _v101);
        const float s2_z = __fmaf_rn(1.0f, 0.0f, _v102);
        out[8] = s2_x; out[9] = s2_y; out[10] = s2_z; out[11] = 0.05999999865889549f;
        const float _v104 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v105 = __fmaf_rn(F0_r01, 0.0f, _v104);
        const float s3_x = __fmaf_rn(0.0f, -0.11999999731779099f, _v105);
        const float _v107 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v108 = __fmaf_rn(F0_r11, 0.0f, _v107);
        const float s3_y = __fmaf_rn(0.0f, -0.11999999731779099f, _v108);
        const float _v110 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v111 = __fmaf_rn(0.0f, 0.0f, _v110);
        const float s3_z = __fmaf_rn(1.0f, -0.11999999731779099f, _v111);
        out[12] = s3_x; out[13] = s3_y; out[14] = s3_z; out[15] = 0.05999999865889549f;
        const float _v113 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v114 = __fmaf_rn(F0_r01, 0.0f, _v113);
        const float s4_x = __fmaf_rn(0.0f, -0.17000000178813934f, _v114);
        const float _v116 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v117 = __fmaf_rn(F0_r11, 0.0f, _v116);
        const float s4_y = __fmaf_rn(0.0f, -0.17000000178813934f, _v117);
        const float _v119 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v120 = __fmaf_rn(0.0f, 0.0f, _v119);
        const float s4_z = __fmaf_rn(1.0f, -0.17000000178813934f, _v120);
        out[16] = s4_x; out[17] = s4_y; out[18] = s4_z; out[19] = 0.05999999865889549f;
        const float _v122 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v123 = __fmaf_rn(F1_r01, 0.0f, _v122);
        const float s5_x = __fmaf_rn(F1_r02, 0.029999999329447746f, _v123);
        const float _v125 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v126 = __fmaf_rn(F1_r11, 0.0f, _v125);
        const float s5_y = __fmaf_rn(F1_r12, 0.029999999329447746f, _v126);
        const float _v128 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v129 = __fmaf_rn(F1_r21, 0.0f, _v128);
        const float s5_z = __fmaf_rn(0.0f, 0.029999999329447746f, _v129);
        out[20] = s5_x; out[21] = s5_y; out[22] = s5_z; out[23] = 0.05999999865889549f;
        const float _v131 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v132 = __fmaf_rn(F1_r01, 0.0f, _v131);
        const float s6_x = __fmaf_rn(F1_r02, 0.07999999821186066f, _v132);
        const float _v134 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v135 = __fmaf_rn(F1_r11, 0.0f, _v134);
        const float s6_y = __fmaf_rn(F1_r12, 0.07999999821186066f, _v135);
        const float _v137 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v138 = __fmaf_rn(F1_r21, 0.0f, _v137);
        const float s6_z = __fmaf_rn(0.0f, 0.07999999821186066f, _v138);
        out[24] = s6_x; out[25] = s6_y; out[26] = s6_z; out[27] = 0.05999999865889549f;
        const float _v140 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v141 = __fmaf_rn(F1_r01, -0.11999999731779099f, _v140);
        const float s7_x = __fmaf_rn(F1_r02, 0.0f, _v141);
        const float _v143 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v144 = __fmaf_rn(F1_r11, -0.11999999731779099f, _v143);
        const float s7_y = __fmaf_rn(F1_r12, 0.0f, _v144);
        const float _v146 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v147 = __fmaf_rn(F1_r21, -0.11999999731779099f, _v146);
        const float s7_z = __fmaf_rn(0.0f, 0.0f, _v147);
        out[28] = s7_x; out[29] = s7_y; out[30] = s7_z; out[31] = 0.05999999865889549f;
        const float _v149 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v150 = __fmaf_rn(F1_r01, -0.17000000178813934f, _v149);
        const float s8_x = __fmaf_rn(F1_r02, 0.0f, _v150);
        const float _v152 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v153 = __fmaf_rn(F1_r11, -0.17000000178813934f, _v152);
        const float s8_y = __fmaf_rn(F1_r12, 0.0f, _v153);
        const float _v155 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v156 = __fmaf_rn(F1_r21, -0.17000000178813934f, _v155);
        const float s8_z = __fmaf_rn(0.0f, 0.0f, _v156);
        out[32] = s8_x; out[33] = s8_y; out[34] = s8_z; out[35] = 0.05999999865889549f;
        const float _v158 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v159 = __fmaf_rn(F2_r01, 0.0f, _v158);
        const float s9_x = __fmaf_rn(F2_r02, -0.10000000149011612f, _v159);
        const float _v161 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v162 = __fmaf_rn(F2_r11, 0.0f, _v161);
        const float s9_y = __fmaf_rn(F2_r12, -0.10000000149011612f, _v162);
        const float _v164 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v165 = __fmaf_rn(F2_r21, 0.0f, _v164);
        const float s9_z = __fmaf_rn(F2_r22, -0.10000000149011612f, _v165);
        out[36] = s9_x; out[37] = s9_y; out[38] = s9_z; out[39] = 0.05999999865889549f;
        const float _v167 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v168 = __fmaf_rn(F2_r01, 0.0f, _v167);
        const float s10_x = __fmaf_rn(F2_r02, -0.05999999865889549f, _v168);
        const float _v170 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v171 = __fmaf_rn(F2_r11, 0.0f, _v170);
        const float s10_y = __fmaf_rn(F2_r12, -0.05999999865889549f, _v171);
        const float _v173 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v174 = __fmaf_rn(F2_r21, 0.0f, _v173);
        const float s10_z = __fmaf_rn(F2_r22, -0.05999999865889549f, _v174);
        out[40] = s10_x; out[41] = s10_y; out[42] = s10_z; out[43] = 0.05000000074505806f;
        const float _v176 = __fmaf_rn(F2_r00, 0.07999999821186066f, F2_t0);
        const float _v177 = __fmaf_rn(F2_r01, 0.05999999865889549f, _v176);
        const float s11_x = __fmaf_rn(F2_r02, 0.0f, _v177);
        const float _v179 = __fmaf_rn(F2_r10, 0.07999999821186066f, F2_t1);
        const float _v180 = __fmaf_rn(F2_r11, 0.05999999865889549f, _v179);
        const float s11_y = __fmaf_rn(F2_r12, 0.0f, _v180);
        const float _v182 = __fmaf_rn(F2_r20, 0.07999999821186066f, F2_t2);
        const float _v183 = __fmaf_rn(F2_r21, 0.05999999865889549f, _v182);
        const float s11_z = __fmaf_rn(F2_r22, 0.0f, _v183);
        out[44] = s11_x; out[45] = s11_y; out[46] = s11_z; out[47] = 0.054999999701976776f;
        const float _v185 = __fmaf_rn(F2_r00, 0.07999999821186066f, F2_t0);
        const float _v186 = __fmaf_rn(F2_r01, 0.019999999552965164f, _v185);
        const float s12_x = __fmaf_rn(F2_r02, 0.0f, _v186);
        const float _v188 = __fmaf_rn(F2_r10, 0.07999999821186066f, F2_t1);
        const float _v189 = __fmaf_rn(F2_r11, 0.019999999552965164f, _v188);
        const float s12_y = __fmaf_rn(F2_r12, 0.0f, _v189);
        const float _v191 = __fmaf_rn(F2_r20, 0.07999999821186066f, F2_t2);
        const float _v192 = __fmaf_rn(F2_r21, 0.019999999552965164f, _v191);
        const float s12_z = __fmaf_rn(F2_r22, 0.0f, _v192);
        out[48] = s12_x; out[49] = s12_y; out[50] = s12_z; out[51] = 0.054999999701976776f;
        const float _v194 = __fmaf_rn(F3_r00, -0.07999999821186066f, F3_t0);
        const float _v195 = __fmaf_rn(F3_r01, 0.0949999988079071f, _v194);
        const float s13_x = __fmaf_rn(F3_r02, 0.0f, _v195);
        const float _v197 = __fmaf_rn(F3_r10, -0.07999999821186066f, F3_t1);
        const float _v198 = __fmaf_rn(F3_r11, 0.0949999988079071f, _v197);
        const float s13_y = __fmaf_rn(F3_r12, 0.0f, _v198);
        const float _v200 = __fmaf_rn(F3_r20, -0.07999999821186066f, F3_t2);
        const float _v201 = __fmaf_rn(F3_r21, 0.0949999988079071f, _v200);
        const float s13_z = __fmaf_rn(F3_r22, 0.0f, _v201);
        out[52] = s13_x; out[53] = s13_y; out[54] = s13_z; out[55] = 0.05999999865889549f;
        const float _v203 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v204 = __fmaf_rn(F3_r01, 0.0f, _v203);
        const float s14_x = __fmaf_rn(F3_r02, 0.019999999552965164f, _v204);
        const float _v206 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v207 = __fmaf_rn(F3_r11, 0.0f, _v206);
        const float s14_y = __fmaf_rn(F3_r12, 0.019999999552965164f, _v207);
        const float _v209 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v210 = __fmaf_rn(F3_r21, 0.0f, _v209);
        const float s14_z = __fmaf_rn(F3_r22, 0.019999999552965164f, _v210);
        out[56] = s14_x; out[57] = s14_y; out[58] = s14_z; out[59] = 0.054999999701976776f;
        const float _v212 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v213 = __fmaf_rn(F3_r01, 0.0f, _v212);
        const float s15_x = __fmaf_rn(F3_r02, 0.05999999865889549f, _v213);
        const float _v215 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v216 = __fmaf_rn(F3_r11, 0.0f, _v215);
        const float s15_y = __fmaf_rn(F3_r12, 0.05999999865889549f, _v216);
        const float _v218 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v219 = __fmaf_rn(F3_r21, 0.0f, _v218);
        const float s15_z = __fmaf_rn(F3_r22, 0.05999999865889549f, _v219);
        out[60] = s15_x; out[61] = s15_y; out[62] = s15_z; out[63] = 0.054999999701976776f;
        const float _v221 = __fmaf_rn(F3_r00, -0.07999999821186066f, F3_t0);
        const float _v222 = __fmaf_rn(F3_r01, 0.05999999865889549f, _v221);
        const float s16_x = __fmaf_rn(F3_r02, 0.0f, _v222);
        const float _v224 = __fmaf_rn(F3_r10, -0.07999999821186066f, F3_t1);
        const float _v225 = __fmaf_rn(F3_r11, 0.05999999865889549f, _v224);
        const float s16_y = __fmaf_rn(F3_r12, 0.0f, _v225);
        const float _v227 = __fmaf_rn(F3_r20, -0.07999999821186066f, F3_t2);
        const float _v228 = __fmaf_rn(F3_r21, 0.05999999865889549f, _v227);
        const float s16_z = __fmaf_rn(F3_r22, 0.0f, _v228);
        out[64] = s16_x; out[65] = s16_y; out[66] = s16_z; out[67] = 0.054999999701976776f;
        const float _v230 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v231 = __fmaf_rn(F4_r01, 0.054999999701976776f, _v230);
        const float s17_x = __fmaf_rn(F4_r02, 0.0f, _v231);
        const float _v233 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v234 = __fmaf_rn(F4_r11, 0.054999999701976776f, _v233);
        const float s17_y = __fmaf_rn(F4_r12, 0.0f, _v234);
        const float _v236 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v237 = __fmaf_rn(F4_r21, 0.054999999701976776f, _v236);
        const float s17_z = __fmaf_rn(F4_r22, 0.0f, _v237);
        out[68] = s17_x; out[69] = s17_y; out[70] = s17_z; out[71] = 0.05999999865889549f;
        const float _v239 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v240 = __fmaf_rn(F4_r01, 0.07500000298023224f, _v239);
        const float s18_x = __fmaf_rn(F4_r02, 0.0f, _v240);
        const float _v242 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v243 = __fmaf_rn(F4_r11, 0.07500000298023224f, _v242);
        const float s18_y = __fmaf_rn(F4_r12, 0.0f, _v243);
        const float _v245 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v246 = __fmaf_rn(F4_r21, 0.07500000298023224f, _v245);
        const float s18_z = __fmaf_rn(F4_r22, 0.0f, _v246);
        out[72] = s18_x; out[73] = s18_y; out[74] = s18_z; out[75] = 0.05999999865889549f;
        const float _v248 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v249 = __fmaf_rn(F4_r01, 0.0f, _v248);
        const float s19_x = __fmaf_rn(F4_r02, -0.2199999988079071f, _v249);
        const float _v251 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v252 = __fmaf_rn(F4_r11, 0.0f, _v251);
        const float s19_y = __fmaf_rn(F4_r12, -0.2199999988079071f, _v252);
        const float _v254 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v255 = __fmaf_rn(F4_r21, 0.0f, _v254);
        const float s19_z = __fmaf_rn(F4_r22, -0.2199999988079071f, _v255);
        out[76] = s19_x; out[77] = s19_y; out[78] = s19_z; out[79] = 0.05999999865889549f;
        const float _v257 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v258 = __fmaf_rn(F4_r01, 0.05000000074505806f, _v257);
        const float s20_x = __fmaf_rn(F4_r02, -0.18000000715255737f, _v258);
        const float _v260 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v261 = __fmaf_rn(F4_r11, 0.05000000074505806f, _v260);
        const float s20_y = __fmaf_rn(F4_r12, -0.18000000715255737f, _v261);
        const float _v263 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v264 = __fmaf_rn(F4_r21, 0.05000000074505806f, _v263);
        const float s20_z = __fmaf_rn(F4_r22, -0.18000000715255737f, _v264);
        out[80] = s20_x; out[81] = s20_y; out[82] = s20_z; out[83] = 0.05000000074505806f;
        const float _v266 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v267 = __fmaf_rn(F4_r01, 0.07999999821186066f, _v266);
        const float s21_x = __fmaf_rn(F4_r02, -0.14000000059604645f, _v267);
        const float _v269 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v270 = __fmaf_rn(F4_r11, 0.07999999821186066f, _v269);
        const float s21_y = __fmaf_rn(F4_r12, -0.14000000059604645f, _v270);
        const float _v272 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v273 = __fmaf_rn(F4_r21, 0.07999999821186066f, _v272);
        const float s21_z = __fmaf_rn(F4_r22, -0.14000000059604645f, _v273);
        out[84] = s21_x; out[85] = s21_y; out[86] = s21_z; out[87] = 0.02500000037252903f;
        const float _v275 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v276 = __fmaf_rn(F4_r01, 0.08500000089406967f, _v275);
        const float s22_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v276);
        const float _v278 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v279 = __fmaf_rn(F4_r11, 0.08500000089406967f, _v278);
        const float s22_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v279);
        const float _v281 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v282 = __fmaf_rn(F4_r21, 0.08500000089406967f, _v281);
        const float s22_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v282);
        out[88] = s22_x; out[89] = s22_y; out[90] = s22_z; out[91] = 0.02500000037252903f;
        const float _v284 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v285 = __fmaf_rn(F4_r01, 0.09000000357627869f, _v284);
        const float s23_x = __fmaf_rn(F4_r02, -0.07999999821186066f, _v285);
        const float _v287 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v288 = __fmaf_rn(F4_r11, 0.09000000357627869f, _v287);
        const float s23_y = __fmaf_rn(F4_r12, -0.07999999821186066f, _v288);
        const float _v290 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v291 = __fmaf_rn(F4_r21, 0.09000000357627869f, _v290);
        const float s23_z = __fmaf_rn(F4_r22, -0.07999999821186066f, _v291);
        out[92] = s23_x; out[93] = s23_y; out[94] = s23_z; out[95] = 0.02500000037252903f;
        const float _v293 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v294 = __fmaf_rn(F4_r01, 0.0949999988079071f, _v293);
        const float s24_x = __fmaf_rn(F4_r02, -0.05000000074505806f, _v294);
        const float _v296 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v297 = __fmaf_rn(F4_r11, 0.0949999988079071f, _v296);
        const float s24_y = __fmaf_rn(F4_r12, -0.05000000074505806f, _v297);
        const float _v299 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v300 = __fmaf_rn(F4_r21, 0.0949999988079071f, _v299);
        const float s24_z = __fmaf_rn(F4_r22, -0.05000000074505806f, _v300);
        out[96] = s24_x; out[97] = s24_y; out[98] = s24_z; out[99] = 0.02500000037252903f;
        const float _v302 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v303 = __fmaf_rn(F4_r01, 0.07999999821186066f, _v302);
        const float s25_x = __fmaf_rn(F4_r02, -0.14000000059604645f, _v303);
        const float _v305 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v306 = __fmaf_rn(F4_r11, 0.07999999821186066f, _v305);
        const float s25_y = __fmaf_rn(F4_r12, -0.14000000059604645f, _v306);
        const float _v308 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v309 = __fmaf_rn(F4_r21, 0.07999999821186066f, _v308);
        const float s25_z = __fmaf_rn(F4_r22, -0.14000000059604645f, _v309);
        out[100] = s25_x; out[101] = s25_y; out[102] = s25_z; out[103] = 0.02500000037252903f;
        const float _v311 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v312 = __fmaf_rn(F4_r01, 0.08500000089406967f, _v311);
        const float s26_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v312);
        const float _v314 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v315 = __fmaf_rn(F4_r11, 0.08500000089406967f, _v314);
        const float s26_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v315);
        const float _v317 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v318 = __fmaf_rn(F4_r21, 0.08500000089406967f, _v317);
        const float s26_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v318);
        out[104] = s26_x; out[105] = s26_y; out[106] = s26_z; out[107] = 0.02500000037252903f;
        const float _v320 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v321 = __fmaf_rn(F4_r01, 0.09000000357627869f, _v320);
        const float s27_x = __fmaf_rn(F4_r02, -0.07999999821186066f, _v321);
        const float _v323 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v324 = __fmaf_rn(F4_r11, 0.09000000357627869f, _v323);
        const float s27_y = __fmaf_rn(F4_r12, -0.07999999821186066f, _v324);
        const float _v326 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v327 = __fmaf_rn(F4_r21, 0.09000000357627869f, _v326);
        const float s27_z = __fmaf_rn(F4_r22, -0.07999999821186066f, _v327);
        out[108] = s27_x; out[109] = s27_y; out[110] = s27_z; out[111] = 0.02500000037252903f;
        const float _v329 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v330 = __fmaf_rn(F4_r01, 0.0949999988079071f, _v329);
        const float s28_x = __fmaf_rn(F4_r02, -0.05000000074505806f, _v330);
        const float _v332 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v333 = __fmaf_rn(F4_r11, 0.0949999988079071f, _v332);
        const float s28_y = __fmaf_rn(F4_r12, -0.05000000074505806f, _v333);
        const float _v335 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v336 = __fmaf_rn(F4_r21, 0.0949999988079071f, _v335);
        const float s28_z = __fmaf_rn(F4_r22, -0.05000000074505806f, _v336);
        out[112] = s28_x; out[113] = s28_y; out[114] = s28_z; out[115] = 0.02500000037252903f;
        const float _v338 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
        const float _v339 = __fmaf_rn(F5_r01, 0.0f, _v338);
        const float s29_x = __fmaf_rn(F5_r02, 0.0f, _v339);
        const float _v341 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
        const float _v342 = __fmaf_rn(F5_r11, 0.0f, _v341);
        const float s29_y = __fmaf_rn(F5_r12, 0.0f, _v342);
        const float _v344 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
        const float _v345 = __fmaf_rn(F5_r21, 0.0f, _v344);
        const float s29_z = __fmaf_rn(F5_r22, 0.0f, _v345);
        out[116] = s29_x; out[117] = s29_y; out[118] = s29_z; out[119] = 0.05000000074505806f;
        const float _v347 = __fmaf_rn(F5_r00, 0.07999999821186066f, F5_t0);
        const float _v348 = __fmaf_rn(F5_r01, -0.009999999776482582f, _v347);
        const float s30_x = __fmaf_rn(F5_r02, 0.0f, _v348);
        const float _v350 = __fmaf_rn(F5_r10, 0.07999999821186066f, F5_t1);
        const float _v351 = __fmaf_rn(F5_r11, -0.009999999776482582f, _v350);
        const float s30_y = __fmaf_rn(F5_r12, 0.0f, _v351);
        const float _v353 = __fmaf_rn(F5_r20, 0.07999999821186066f, F5_t2);
        const float _v354 = __fmaf_rn(F5_r21, -0.009999999776482582f, _v353);
        const float s30_z = __fmaf_rn(F5_r22, 0.0f, _v354);
        out[120] = s30_x; out[121] = s30_y; out[122] = s30_z; out[123] = 0.05000000074505806f;
        const float _v356 = __fmaf_rn(F5_r00, 0.07999999821186066f, F5_t0);
        const float _v357 = __fmaf_rn(F5_r01, 0.03500000014901161f, _v356);
        const float s31_x = __fmaf_rn(F5_r02, 0.0f, _v357);
        const float _v359 = __fmaf_rn(F5_r10, 0.07999999821186066f, F5_t1);
        const float _v360 = __fmaf_rn(F5_r11, 0.03500000014901161f, _v359);
        const float s31_y = __fmaf_rn(F5_r12, 0.0f, _v360);
        const float _v362 = __fmaf_rn(F5_r20, 0.07999999821186066f, F5_t2);
        const float _v363 = __fmaf_rn(F5_r21, 0.03500000014901161f, _v362);
        const float s31_z = __fmaf_rn(F5_r22, 0.0f, _v363);
        out[124] = s31_x; out[125] = s31_y; out[126] = s31_z; out[127] = 0.052000001072883606f;
        const float _v365 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
        const float _v366 = __fmaf_rn(F6_r01, 0.0f, _v365);
        const float s32_x = __fmaf_rn(F6_r02, 0.07000000029802322f, _v366);
        const float _v368 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
        const float _v369 = __fmaf_rn(F6_r11, 0.0f, _v368);
        const float s32_y = __fmaf_rn(F6_r12, 0.07000000029802322f, _v369);
        const float _v371 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
        const float _v372 = __fmaf_rn(F6_r21, 0.0f, _v371);
        const float s32_z = __fmaf_rn(F6_r22, 0.07000000029802322f, _v372);
        out[128] = s32_x; out[129] = s32_y; out[130] = s32_z; out[131] = 0.05000000074505806f;
        const float _v374 = __fmaf_rn(F6_r00, 0.019999999552965164f, F6_t0);
        const float _v375 = __fmaf_rn(F6_r01, 0.03999999910593033f, _v374);
        const float s33_x = __fmaf_rn(F6_r02, 0.07999999821186066f, _v375);
        const float _v377 = __fmaf_rn(F6_r10, 0.019999999552965164f, F6_t1);
        const float _v378 = __fmaf_rn(F6_r11, 0.03999999910593033f, _v377);
        const float s33_y = __fmaf_rn(F6_r12, 0.07999999821186066f, _v378);
        const float _v380 = __fmaf_rn(F6_r20, 0.019999999552965164f, F6_t2);
        const float _v381 = __fmaf_rn(F6_r21, 0.03999999910593033f, _v380);
        const float s33_z = __fmaf_rn(F6_r22, 0.07999999821186066f, _v381);
        out[132] = s33_x; out[133] = s33_y; out[134] = s33_z; out[135] = 0.02500000037252903f;
        const float _v383 = __fmaf_rn(F6_r00, 0.03999999910593033f, F6_t0);
        const float _v384 = __fmaf_rn(F6_r01, 0.019999999552965164f, _v383);
        const float s34_x = __fmaf_rn(F6_r02, 0.07999999821186066f, _v384);
        const float _v386 = __fmaf_rn(F6_r10, 0.03999999910593033f, F6_t1);
        const float _v387 = __fmaf_rn(F6_r11, 0.019999999552965164f, _v386);
        const float s34_y = __fmaf_rn(F6_r12, 0.07999999821186066f, _v387);
        const float _v389 = __fmaf_rn(F6_r20, 0.03999999910593033f, F6_t2);
        const float _v390 = __fmaf_rn(F6_r21, 0.019999999552965164f, _v389);
        const float s34_z = __fmaf_rn(F6_r22, 0.07999999821186066f, _v390);
        out[136] = s34_x; out[137] = s34_y; out[138] = s34_z; out[139] = 0.02500000037252903f;
        const float _v392 = __fmaf_rn(F6_r00, 0.03999999910593033f, F6_t0);
        const float _v393 = __fmaf_rn(F6_r01, 0.05999999865889549f, _v392);
        const float s35_x = __fmaf_rn(F6_r02, 0.08500000089406967f, _v393);
        const float _v395 = __fmaf_rn(F6_r10, 0.03999999910593033f, F6_t1);
        const float _v396 = __fmaf_rn(F6_r11, 0.05999999865889549f, _v395);
        const float s35_y = __fmaf_rn(F6_r12, 0.08500000089406967f, _v396);
        const float _v398 = __fmaf_rn(F6_r20, 0.03999999910593033f, F6_t2);
        const float _v399 = __fmaf_rn(F6_r21, 0.05999999865889549f, _v398);
        const float s35_z = __fmaf_rn(F6_r22, 0.08500000089406967f, _v399);
        out[140] = s35_x; out[141] = s35_y; out[142] = s35_z; out[143] = 0.019999999552965164f;
        const float _v401 = __fmaf_rn(F6_r00, 0.05999999865889549f, F6_t0);
        const float _v402 = __fmaf_rn(F6_r01, 0.03999999910593033f, _v401);
        const float s36_x = __fmaf_rn(F6_r02, 0.08500000089406967f, _v402);
        const float _v404 = __fmaf_rn(F6_r10, 0.05999999865889549f, F6_t1);
        const float _v405 = __fmaf_rn(F6_r11, 0.03999999910593033f, _v404);
        const float s36_y = __fmaf_rn(F6_r12, 0.08500000089406967f, _v405);
        const float _v407 = __fmaf_rn(F6_r20, 0.05999999865889549f, F6_t2);
        const float _v408 = __fmaf_rn(F6_r21, 0.03999999910593033f, _v407);
        const float s36_z = __fmaf_rn(F6_r22, 0.08500000089406967f, _v408);
        out[144] = s36_x; out[145] = s36_y; out[146] = s36_z; out[147] = 0.019999999552965164f;
        const float _v410 = __fmaf_rn(F6_r00, -0.0530330091714859f, F6_t0);
        const float _v411 = __fmaf_rn(F6_r01, -0.0530330091714859f, _v410);
        const float s37_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v411);
        const float _v413 = __fmaf_rn(F6_r10, -0.0530330091714859f, F6_t1);
        const float _v414 = __fmaf_rn(F6_r11, -0.0530330091714859f, _v413);
        const float s37_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v414);
        const float _v416 = __fmaf_rn(F6_r20, -0.0530330091714859f, F6_t2);
        const float _v417 = __fmaf_rn(F6_r21, -0.0530330091714859f, _v416);
        const float s37_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v417);
        out[148] = s37_x; out[149] = s37_y; out[150] = s37_z; out[151] = 0.02800000086426735f;
        const float _v419 = __fmaf_rn(F6_r00, -0.03181980550289154f, F6_t0);
        const float _v420 = __fmaf_rn(F6_r01, -0.03181980550289154f, _v419);
        const float s38_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v420);
        const float _v422 = __fmaf_rn(F6_r10, -0.03181980550289154f, F6_t1);
        const float _v423 = __fmaf_rn(F6_r11, -0.03181980550289154f, _v422);
        const float s38_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v423);
        const float _v425 = __fmaf_rn(F6_r20, -0.03181980550289154f, F6_t2);
        const float _v426 = __fmaf_rn(F6_r21, -0.03181980550289154f, _v425);
        const float s38_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v426);
        out[152] = s38_x; out[153] = s38_y; out[154] = s38_z; out[155] = 0.02800000086426735f;
        const float _v428 = __fmaf_rn(F6_r00, -0.01060660183429718f, F6_t0);
        const float _v429 = __fmaf_rn(F6_r01, -0.01060660183429718f, _v428);
        const float s39_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v429);
        const float _v431 = __fmaf_rn(F6_r10, -0.01060660183429718f, F6_t1);
        const float _v432 = __fmaf_rn(F6_r11, -0.01060660183429718f, _v431);
        const float s39_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v432);
        const float _v434 = __fmaf_rn(F6_r20, -0.01060660183429718f, F6_t2);
        const float _v435 = __fmaf_rn(F6_r21, -0.01060660183429718f, _v434);
        const float s39_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v435);
        out[156] = s39_x; out[157] = s39_y; out[158] = s39_z; out[159] = 0.02800000086426735f;
        const float _v437 = __fmaf_rn(F6_r00, 0.01060660183429718f, F6_t0);
        const float _v438 = __fmaf_rn(F6_r01, 0.01060660183429718f, _v437);
        const float s40_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v438);
        const float _v440 = __fmaf_rn(F6_r10, 0.01060660183429718f, F6_t1);
        const float _v441 = __fmaf_rn(F6_r11, 0.01060660183429718f, _v440);
        const float s40_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v441);
        const float _v443 = __fmaf_rn(F6_r20, 0.01060660183429718f, F6_t2);
        const float _v444 = __fmaf_rn(F6_r21, 0.01060660183429718f, _v443);
        const float s40_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v444);
        out[160] = s40_x; out[161] = s40_y; out[162] = s40_z; out[163] = 0.02800000086426735f;
        const float _v446 = __fmaf_rn(F6_r00, 0.03181980550289154f, F6_t0);
        const float _v447 = __fmaf_rn(F6_r01, 0.03181980550289154f, _v446);
        const float s41_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v447);
        const float _v449 = __fmaf_rn(F6_r10, 0.03181980550289154f, F6_t1);
        const float _v450 = __fmaf_rn(F6_r11, 0.03181980550289154f, _v449);
        const float s41_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v450);
        const float _v452 = __fmaf_rn(F6_r20, 0.03181980550289154f, F6_t2);
        const float _v453 = __fmaf_rn(F6_r21, 0.03181980550289154f, _v452);
        const float s41_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v453);
        out[164] = s41_x; out[165] = s41_y; out[166] = s41_z; out[167] = 0.02800000086426735f;
        const float _v455 = __fmaf_rn(F6_r00, 0.0530330091714859f, F6_t0);
        const float _v456 = __fmaf_rn(F6_r01, 0.0530330091714859f, _v455);
        const float s42_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v456);
        const float _v458 = __fmaf_rn(F6_r10, 0.0530330091714859f, F6_t1);
        const float _v459 = __fmaf_rn(F6_r11, 0.0530330091714859f, _v458);
        const float s42_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v459);
        const float _v461 = __fmaf_rn(F6_r20, 0.0530330091714859f, F6_t2);
        const float _v462 = __fmaf_rn(F6_r21, 0.0530330091714859f, _v461);
        const float s42_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v462);
        out[168] = s42_x; out[169] = s42_y; out[170] = s42_z; out[171] = 0.02800000086426735f;
        const float _v464 = __fmaf_rn(F6_r00, -0.0530330091714859f, F6_t0);
        const float _v465 = __fmaf_rn(F6_r01, -0.0530330091714859f, _v464);
        const float s43_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v465);
        const float _v467 = __fmaf_rn(F6_r10, -0.0530330091714859f, F6_t1);
        const float _v468 = __fmaf_rn(F6_r11, -0.0530330091714859f, _v467);
        const float s43_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v468);
        const float _v470 = __fmaf_rn(F6_r20, -0.0530330091714859f, F6_t2);
        const float _v471 = __fmaf_rn(F6_r21, -0.0530330091714859f, _v470);
        const float s43_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v471);
        out[172] = s43_x; out[173] = s43_y; out[174] = s43_z; out[175] = 0.026000000536441803f;
        const float _v473 = __fmaf_rn(F6_r00, -0.03181980550289154f, F6_t0);
        const float _v474 = __fmaf_rn(F6_r01, -0.03181980550289154f, _v473);
        const float s44_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v474);
        const float _v476 = __fmaf_rn(F6_r10, -0.03181980550289154f, F6_t1);
        const float _v477 = __fmaf_rn(F6_r11, -0.03181980550289154f, _v476);
        const float s44_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v477);
        const float _v479 = __fmaf_rn(F6_r20, -0.03181980550289154f, F6_t2);
        const float _v480 = __fmaf_rn(F6_r21, -0.03181980550289154f, _v479);
        const float s44_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v480);
        out[176] = s44_x; out[177] = s44_y; out[178] = s44_z; out[179] = 0.026000000536441803f;
        const float _v482 = __fmaf_rn(F6_r00, -0.01060660183429718f, F6_t0);
        const float _v483 = __fmaf_rn(F6_r01, -0.01060660183429718f, _v482);
        const float s45_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v483);
        const float _v485 = __fmaf_rn(F6_r10, -0.01060660183429718f, F6_t1);
        const float _v486 = __fmaf_rn(F6_r11, -0.01060660183429718f, _v485);
        const float s45_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v486);
        const float _v488 = __fmaf_rn(F6_r20, -0.01060660183429718f, F6_t2);
        const float _v489 = __fmaf_rn(F6_r21, -0.01060660183429718f, _v488);
        const float s45_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v489);
        out[180] = s45_x; out[181] = s45_y; out[182] = s45_z; out[183] = 0.026000000536441803f;
        const float _v491 = __fmaf_rn(F6_r00, 0.01060660183429718f, F6_t0);
        const float _v492 = __fmaf_rn(F6_r01, 0.01060660183429718f, _v491);
        const float s46_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v492);
        const float _v494 = __fmaf_rn(F6_r10, 0.01060660183429718f, F6_t1);
        const float _v495 = __fmaf_rn(F6_r11, 0.01060660183429718f, _v494);
        const float s46_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v495);
        const float _v497 = __fmaf_rn(F6_r20, 0.01060660183429718f, F6_t2);
        const float _v498 = __fmaf_rn(F6_r21, 0.01060660183429718f, _v497);
        const float s46_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v498);
        out[184] = s46_x; out[185] = s46_y; out[186] = s46_z; out[187] = 0.026000000536441803f;
        const float _v500 = __fmaf_rn(F6_r00, 0.03181980550289154f, F6_t0);
        const float _v501 = __fmaf_rn(F6_r01, 0.03181980550289154f, _v500);
        const float s47_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v501);
        const float _v503 = __fmaf_rn(F6_r10, 0.03181980550289154f, F6_t1);
        const float _v504 = __fmaf_rn(F6_r11, 0.03181980550289154f, _v503);
        const float s47_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v504);
        const float _v506 = __fmaf_rn(F6_r20, 0.03181980550289154f, F6_t2);
        const float _v507 = __fmaf_rn(F6_r21, 0.03181980550289154f, _v506);
        const float s47_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v507);
        out[188] = s47_x; out[189] = s47_y; out[190] = s47_z; out[191] = 0.026000000536441803f;
        const float _v509 = __fmaf_rn(F6_r00, 0.0530330091714859f, F6_t0);
        const float _v510 = __fmaf_rn(F6_r01, 0.0530330091714859f, _v509);
        const float s48_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v510);
        const float _v512 = __fmaf_rn(F6_r10, 0.0530330091714859f, F6_t1);
        const float _v513 = __fmaf_rn(F6_r11, 0.0530330091714859f, _v512);
        const float s48_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v513);
        const float _v515 = __fmaf_rn(F6_r20, 0.0530330091714859f, F6_t2);
        const float _v516 = __fmaf_rn(F6_r21, 0.0530330091714859f, _v515);
        const float s48_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v516);
        out[192] = s48_x; out[193] = s48_y; out[194] = s48_z; out[195] = 0.026000000536441803f;
        const float _v518 = __fmaf_rn(F6_r00, -0.0530330091714859f, F6_t0);
        const float _v519 = __fmaf_rn(F6_r01, -0.0530330091714859f, _v518);
        const float s49_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v519);
        const float _v521 = __fmaf_rn(F6_r10, -0.0530330091714859f, F6_t1);
        const float _v522 = __fmaf_rn(F6_r11, -0.0530330091714859f, _v521);
        const float s49_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v522);
        const float _v524 = __fmaf_rn(F6_r20, -0.0530330091714859f, F6_t2);
        const float _v525 = __fmaf_rn(F6_r21, -0.0530330091714859f, _v524);
        const float s49_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v525);
        out[196] = s49_x; out[197] = s49_y; out[198] = s49_z; out[199] = 0.024000000208616257f;
        const float _v527 = __fmaf_rn(F6_r00, -0.03181980550289154f, F6_t0);
        const float _v528 = __fmaf_rn(F6_r01, -0.03181980550289154f, _v527);
        const float s50_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v528);
        const float _v530 = __fmaf_rn(F6_r10, -0.03181980550289154f, F6_t1);
        const float _v531 = __fmaf_rn(F6_r11, -0.03181980550289154f, _v530);
        const float s50_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v531);
        const float _v533 = __fmaf_rn(F6_r20, -0.03181980550289154f, F6_t2);
        const float _v534 = __fmaf_rn(F6_r21, -0.03181980550289154f, _v533);
        const float s50_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v534);
        out[200] = s50_x; out[201] = s50_y; out[202] = s50_z; out[203] = 0.024000000208616257f;
        const float _v536 = __fmaf_rn(F6_r00, -0.01060660183429718f, F6_t0);
        const float _v537 = __fmaf_rn(F6_r01, -0.01060660183429718f, _v536);
        const float s51_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v537);
        const float _v539 = __fmaf_rn(F6_r10, -0.01060660183429718f, F6_t1);
        const float _v540 = __fmaf_rn(F6_r11, -0.01060660183429718f, _v539);
        const float s51_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v540);
        const float _v542 = __fmaf_rn(F6_r20, -0.01060660183429718f, F6_t2);
        const float _v543 = __fmaf_rn(F6_r21, -0.01060660183429718f, _v542);
        const float s51_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v543);
        out[204] = s51_x; out[205] = s51_y; out[206] = s51_z; out[207] = 0.024000000208616257f;
        const float _v545 = __fmaf_rn(F6_r00, 0.01060660183429718f, F6_t0);
        const float _v546 = __fmaf_rn(F6_r01, 0.01060660183429718f, _v545);
        const float s52_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v546);
        const float _v548 = __fmaf_rn(F6_r10, 0.01060660183429718f, F6_t1);
        const float _v549 = __fmaf_rn(F6_r11, 0.01060660183429718f, _v548);
        const float s52_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v549);
        const float _v551 = __fmaf_rn(F6_r20, 0.01060660183429718f, F6_t2);
        const float _v552 = __fmaf_rn(F6_r21, 0.01060660183429718f, _v551);
        const float s52_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v552);
        out[208] = s52_x; out[209] = s52_y; out[210] = s52_z; out[211] = 0.024000000208616257f;
        const float _v554 = __fmaf_rn(F6_r00, 0.03181980550289154f, F6_t0);
        const float _v555 = __fmaf_rn(F6_r01, 0.03181980550289154f, _v554);
        const float s53_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v555);
        const float _v557 = __fmaf_rn(F6_r10, 0.03181980550289154f, F6_t1);
        const float _v558 = __fmaf_rn(F6_r11, 0.03181980550289154f, _v557);
        const float s53_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v558);
        const float _v560 = __fmaf_rn(F6_r20, 0.03181980550289154f, F6_t2);
        const float _v561 = __fmaf_rn(F6_r21, 0.03181980550289154f, _v560);
        const float s53_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v561);
        out[212] = s53_x; out[213] = s53_y; out[214] = s53_z; out[215] = 0.024000000208616257f;
        const float _v563 = __fmaf_rn(F6_r00, 0.0530330091714859f, F6_t0);
        const float _v564 = __fmaf_rn(F6_r01, 0.0530330091714859f, _v563);
        const float s54_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v564);
        const float _v566 = __fmaf_rn(F6_r10, 0.0530330091714859f, F6_t1);
        const float _v567 = __fmaf_rn(F6_r11, 0.0530330091714859f, _v566);
        const float s54_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v567);
        const float _v569 = __fmaf_rn(F6_r20, 0.0530330091714859f, F6_t2);
        const float _v570 = __fmaf_rn(F6_r21, 0.0530330091714859f, _v569);
        const float s54_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v570);
        out[216] = s54_x; out[217] = s54_y; out[218] = s54_z; out[219] = 0.024000000208616257f;
        const float _v572 = __fmaf_rn(F6_r00, 0.05656854063272476f, F6_t0);
        const float _v573 = __fmaf_rn(F6_r01, 0.05656854063272476f, _v572);
        const float s55_x = __fmaf_rn(F6_r02, 0.1873999983072281f, _v573);
        const float _v575 = __fmaf_rn(F6_r10, 0.05656854063272476f, F6_t1);
        const float _v576 = __fmaf_rn(F6_r11, 0.05656854063272476f, _v575);
        const float s55_y = __fmaf_rn(F6_r12, 0.1873999983072281f, _v576);
        const float _v578 = __fmaf_rn(F6_r20, 0.05656854063272476f, F6_t2);
        const float _v579 = __fmaf_rn(F6_r21, 0.05656854063272476f, _v578);
        const float s55_z = __fmaf_rn(F6_r22, 0.1873999983072281f, _v579);
        out[220] = s55_x; out[221] = s55_y; out[222] = s55_z; out[223] = 0.012000000104308128f;
        const float _v581 = __fmaf_rn(F6_r00, 0.0516187958419323f, F6_t0);
        const float _v582 = __fmaf_rn(F6_r01, 0.0516187958419323f, _v581);
        const float s56_x = __fmaf_rn(F6_r02, 0.2093999981880188f, _v582);
        const float _v584 = __fmaf_rn(F6_r10, 0.0516187958419323f, F6_t1);
        const float _v585 = __fmaf_rn(F6_r11, 0.0516187958419323f, _v584);
        const float s56_y = __fmaf_rn(F6_r12, 0.2093999981880188f, _v585);
        const float _v587 = __fmaf_rn(F6_r20, 0.0516187958419323f, F6_t2);
        const float _v588 = __fmaf_rn(F6_r21, 0.0516187958419323f, _v587);
        const float s56_z = __fmaf_rn(F6_r22, 0.2093999981880188f, _v588);
        out[224] = s56_x; out[225] = s56_y; out[226] = s56_z; out[227] = 0.012000000104308128f;
        const float _v590 = __fmaf_rn(F6_r00, -0.05656854063272476f, F6_t0);
        const float _v591 = __fmaf_rn(F6_r01, -0.05656854063272476f, _v590);
        const float s57_x = __fmaf_rn(F6_r02, 0.1873999983072281f, _v591);
        const float _v593 = __fmaf_rn(F6_r10, -0.05656854063272476f, F6_t1);
        const float _v594 = __fmaf_rn(F6_r11, -0.05656854063272476f, _v593);
        const float s57_y = __fmaf_rn(F6_r12, 0.1873999983072281f, _v594);
        const float _v596 = __fmaf_rn(F6_r20, -0.05656854063272476f, F6_t2);
        const float _v597 = __fmaf_rn(F6_r21, -0.05656854063272476f, _v596);
        const float s57_z = __fmaf_rn(F6_r22, 0.1873999983072281f, _v597);
        out[228] = s57_x; out[229] = s57_y; out[230] = s57_z; out[231] = 0.012000000104308128f;
        const float _v599 = __fmaf_rn(F6_r00, -0.0516187958419323f, F6_t0);
        const float _v600 = __fmaf_rn(F6_r01, -0.0516187958419323f, _v599);
        const float s58_x = __fmaf_rn(F6_r02, 0.2093999981880188f, _v600);
        const float _v602 = __fmaf_rn(F6_r10, -0.0516187958419323f, F6_t1);
        const float _v603 = __fmaf_rn(F6_r11, -0.0516187958419323f, _v602);
        const float s58_y = __fmaf_rn(F6_r12, 0.2093999981880188f, _v603);
        const float _v605 = __fmaf_rn(F6_r20, -0.0516187958419323f, F6_t2);
        const float _v606 = __fmaf_rn(F6_r21, -0.0516187958419323f, _v605);
        const float s58_z = __fmaf_rn(F6_r22, 0.2093999981880188f, _v606);
        out[232] = s58_x; out[233] = s58_y; out[234] = s58_z; out[235] = 0.012000000104308128f;
        const float _v608 = __fmaf_rn(F6_r00, -0.05409367009997368f, F6_t0);
        const float _v609 = __fmaf_rn(F6_r01, -0.05409367009997368f, _v608);
        const float s59_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v609);
        const float _v611 = __fmaf_rn(F6_r10, -0.05409367009997368f, F6_t1);
        const float _v612 = __fmaf_rn(F6_r11, -0.05409367009997368f, _v611);
        const float s59_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v612);
        const float _v614 = __fmaf_rn(F6_r20, -0.05409367009997368f, F6_t2);
        const float _v615 = __fmaf_rn(F6_r21, -0.05409367009997368f, _v614);
        const float s59_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v615);
        out[236] = s59_x; out[237] = s59_y; out[238] = s59_z; out[239] = 0.023543396964669228f;
        const float _v617 = __fmaf_rn(F6_r00, 0.05409367009997368f, F6_t0);
        const float _v618 = __fmaf_rn(F6_r01, 0.05409367009997368f, _v617);
        const float s60_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v618);
        const float _v620 = __fmaf_rn(F6_r10, 0.05409367009997368f, F6_t1);
        const float _v621 = __fmaf_rn(F6_r11, 0.05409367009997368f, _v620);
        const float s60_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v621);
        const float _v623 = __fmaf_rn(F6_r20, 0.05409367009997368f, F6_t2);
        const float _v624 = __fmaf_rn(F6_r21, 0.05409367009997368f, _v623);
        const float s60_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v624);
        out[240] = s60_x; out[241] = s60_y; out[242] = s60_z; out[243] = 0.023543396964669228f;
        const float _v626 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
        const float _v627 = __fmaf_rn(F6_r01, 0.0f, _v626);
        const float s61_x = __fmaf_rn(F6_r02, 0.12920139729976654f, _v627);
        const float _v629 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
        const float _v630 = __fmaf_rn(F6_r11, 0.0f, _v629);
        const float s61_y = __fmaf_rn(F6_r12, 0.12920139729976654f, _v630);
        const float _v632 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
        const float _v633 = __fmaf_rn(F6_r21, 0.0f, _v632);
        const float s61_z = __fmaf_rn(F6_r22, 0.12920139729976654f, _v633);
        out[244] = s61_x; out[245] = s61_y; out[246] = s61_z; out[247] = 0.10398600995540619f;
        const float _v635 = __fmaf_rn(F6_r00, 0.015300550498068333f, F6_t0);
        const float _v636 = __fmaf_rn(F6_r01, 0.015300550498068333f, _v635);
        const float s62_x = __fmaf_rn(F6_r02, 0.07459016144275665f, _v636);
        const float _v638 = __fmaf_rn(F6_r10, 0.015300550498068333f, F6_t1);
        const float _v639 = __fmaf_rn(F6_r11, 0.015300550498068333f, _v638);
        const float s62_y = __fmaf_rn(F6_r12, 0.07459016144275665f, _v639);
        const float _v641 = __fmaf_rn(F6_r20, 0.015300550498068333f, F6_t2);
        const float _v642 = __fmaf_rn(F6_r21, 0.015300550498068333f, _v641);
        const float s62_z = __fmaf_rn(F6_r22, 0.07459016144275665f, _v642);
        out[248] = s62_x; out[249] = s62_y; out[250] = s62_z; out[251] = 0.07211975008249283f;
        const float _v644 = __fmaf_rn(F5_r00, 0.04243096336722374f, F5_t0);
        const float _v645 = __fmaf_rn(F5_r01, 0.014447699300944805f, _v644);
        const float s63_x = __fmaf_rn(F5_r02, 0.0f, _v645);
        const float _v647 = __fmaf_rn(F5_r10, 0.04243096336722374f, F5_t1);
        const float _v648 = __fmaf_rn(F5_r11, 0.014447699300944805f, _v647);
        const float s63_y = __fmaf_rn(F5_r12, 0.0f, _v648);
        const float _v650 = __fmaf_rn(F5_r20, 0.04243096336722374f, F5_t2);
        const float _v651 = __fmaf_rn(F5_r21, 0.014447699300944805f, _v650);
        const float s63_z = __fmaf_rn(F5_r22, 0.0f, _v651);
        out[252] = s63_x; out[253] = s63_y; out[254] = s63_z; out[255] = 0.09482324123382568f;
        const float _v653 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v654 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v653);
        const float s64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v654);
        const float _v656 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v657 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v656);
        const float s64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v657);
        const float _v659 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v660 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v659);
        const float s64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v660);
        out[256] = s64_x; out[257] = s64_y; out[258] = s64_z; out[259] = 0.17621639370918274f;
        const float _v662 = __fmaf_rn(F3_r00, -0.04144999757409096f, F3_t0);
        const float _v663 = __fmaf_rn(F3_r01, 0.04922187328338623f, _v662);
        const float s65_x = __fmaf_rn(F3_r02, 0.02891250140964985f, _v663);
        const float _v665 = __fmaf_rn(F3_r10, -0.04144999757409096f, F3_t1);
        const float _v666 = __fmaf_rn(F3_r11, 0.04922187328338623f, _v665);
        const float s65_y = __fmaf_rn(F3_r12, 0.02891250140964985f, _v666);
        const float _v668 = __fmaf_rn(F3_r20, -0.04144999757409096f, F3_t2);
        const float _v669 = __fmaf_rn(F3_r21, 0.04922187328338623f, _v668);
        const float s65_z = __fmaf_rn(F3_r22, 0.02891250140964985f, _v669);
        out[260] = s65_x; out[261] = s65_y; out[262] = s65_z; out[263] = 0.1264655739068985f;
        const float _v671 = __fmaf_rn(F2_r00, 0.038585785776376724f, F2_t0);
        const float _v672 = __fmaf_rn(F2_r01, 0.028939340263605118f, _v671);
        const float s66_x = __fmaf_rn(F2_r02, -0.05176776647567749f, _v672);
        const float _v674 = __fmaf_rn(F2_r10, 0.038585785776376724f, F2_t1);
        const float _v675 = __fmaf_rn(F2_r11, 0.028939340263605118f, _v674);
        const float s66_y = __fmaf_rn(F2_r12, -0.05176776647567749f, _v675);
        const float _v677 = __fmaf_rn(F2_r20, 0.038585785776376724f, F2_t2);
        const float _v678 = __fmaf_rn(F2_r21, 0.028939340263605118f, _v677);
        const float s66_z = __fmaf_rn(F2_r22, -0.05176776647567749f, _v678);
        out[264] = s66_x; out[265] = s66_y; out[266] = s66_z; out[267] = 0.12821067869663239f;
        const float _v680 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v681 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v680);
        const float s67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v681);
        const float _v683 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v684 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v683);
        const float s67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v684);
        const float _v686 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v687 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v686);
        const float s67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v687);
        out[268] = s67_x; out[269] = s67_y; out[270] = s67_z; out[271] = 0.15394146740436554f;
        const float _v689 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v690 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v689);
        const float s68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v690);
        const float _v692 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v693 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v692);
        const float s68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v693);
        const float _v695 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v696 = __fmaf_rn(0.0f, -0.03999999910593033f, _v695);
        const float s68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v696);
        out[272] = s68_x; out[273] = s68_y; out[274] = s68_z; out[275] = 0.15394146740436554f;
        const float _v698 = __fmaf_rn(1.0f, 0.0f, 0.0f);
        const float _v699 = __fmaf_rn(0.0f, 0.0f, _v698);
        const float s69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v699);
        const float _v701 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v702 = __fmaf_rn(1.0f, 0.0f, _v701);
        const float s69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v702);
        const float _v704 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v705 = __fmaf_rn(0.0f, 0.0f, _v704);
        const float s69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v705);
        out[276] = s69_x; out[277] = s69_y; out[278] = s69_z; out[279] = 0.07999999821186066f;
    }

    // fine spheres [57, 58] (panda_rightfinger)
    static __device__ __noinline__ void fine_0(const float F6_r00, const float F6_r01, const float F6_r02, const float F6_r10, const float F6_r11, const float F6_r12, const float F6_r20, const float F6_r21, const float F6_r22, const float F6_t0, const float F6_t1, const float F6_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F6_r00, -0.05656854063272476f, F6_t0);
        const float _v100001 = __fmaf_rn(F6_r01, -0.05656854063272476f, _v100000);
        const float s0_x = __fmaf_rn(F6_r02, 0.1873999983072281f, _v100001);
        const float _v100003 = __fmaf_rn(F6_r10, -0.05656854063272476f, F6_t1);
        const float _v100004 = __fmaf_rn(F6_r11, -0.05656854063272476f, _v100003);
        const float s0_y = __fmaf_rn(F6_r12, 0.1873999983072281f, _v100004);
        const float _v100006 = __fmaf_rn(F6_r20, -0.05656854063272476f, F6_t2);
        const float _v100007 = __fmaf_rn(F6_r21, -0.05656854063272476f, _v100006);
        const float s0_z = __fmaf_rn(F6_r22, 0.1873999983072281f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.012000000104308128f);
        const float _v100009 = __fmaf_rn(F6_r00, -0.0516187958419323f, F6_t0);
        const float _v100010 = __fmaf_rn(F6_r01, -0.0516187958419323f, _v100009);
        const float s1_x = __fmaf_rn(F6_r02, 0.2093999981880188f, _v100010);
        const float _v100012 = __fmaf_rn(F6_r10, -0.0516187958419323f, F6_t1);
        const float _v100013 = __fmaf_rn(F6_r11, -0.0516187958419323f, _v100012);
        const float s1_y = __fmaf_rn(F6_r12, 0.2093999981880188f, _v100013);
        const float _v100015 = __fmaf_rn(F6_r20, -0.0516187958419323f, F6_t2);
        const float _v100016 = __fmaf_rn(F6_r21, -0.0516187958419323f, _v100015);
        const float s1_z = __fmaf_rn(F6_r22, 0.2093999981880188f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.012000000104308128f);
    }
    // fine spheres [55, 56] (panda_leftfinger)
    static __device__ __noinline__ void fine_1(const float F6_r00, const float F6_r01, const float F6_r02, const float F6_r10, const float F6_r11, const float F6_r12, const float F6_r20, const float F6_r21, const float F6_r22, const float F6_t0, const float F6_t1, const float F6_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F6_r00, 0.05656854063272476f, F6_t0);
        const float _v100001 = __fmaf_rn(F6_r01, 0.05656854063272476f, _v100000);
        const float s0_x = __fmaf_rn(F6_r02, 0.1873999983072281f, _v100001);
        const float _v100003 = __fmaf_rn(F6_r10, 0.05656854063272476f, F6_t1);
        const float _v100004 = __fmaf_rn(F6_r11, 0.05656854063272476f, _v100003);
        const float s0_y = __fmaf_rn(F6_r12, 0.1873999983072281f, _v100004);
        const float _v100006 = __fmaf_rn(F6_r20, 0.05656854063272476f, F6_t2);
        const float _v100007 = __fmaf_rn(F6_r21, 0.05656854063272476f, _v100006);
        const float s0_z = __fmaf_rn(F6_r22, 0.1873999983072281f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.012000000104308128f);
        const float _v100009 = __fmaf_rn(F6_r00, 0.0516187958419323f, F6_t0);
        const float _v100010 = __fmaf_rn(F6_r01, 0.0516187958419323f, _v100009);
        const float s1_x = __fmaf_rn(F6_r02, 0.2093999981880188f, _v100010);
        const float _v100012 = __fmaf_rn(F6_r10, 0.0516187958419323f, F6_t1);
        const float _v100013 = __fmaf_rn(F6_r11, 0.0516187958419323f, _v100012);
        const float s1_y = __fmaf_rn(F6_r12, 0.2093999981880188f, _v100013);
        const float _v100015 = __fmaf_rn(F6_r20, 0.0516187958419323f, F6_t2);
        const float _v100016 = __fmaf_rn(F6_r21, 0.0516187958419323f, _v100015);
        const float s1_z = __fmaf_rn(F6_r22, 0.2093999981880188f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.012000000104308128f);
    }
    // fine spheres [37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 50, 51, 52, 53, 54] (panda_hand)
    static __device__ __noinline__ void fine_2(const float F6_r00, const float F6_r01, const float F6_r02, const float F6_r10, const float F6_r11, const float F6_r12, const float F6_r20, const float F6_r21, const float F6_r22, const float F6_t0, const float F6_t1, const float F6_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F6_r00, -0.0530330091714859f, F6_t0);
        const float _v100001 = __fmaf_rn(F6_r01, -0.0530330091714859f, _v100000);
        const float s0_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v100001);
        const float _v100003 = __fmaf_rn(F6_r10, -0.0530330091714859f, F6_t1);
        const float _v100004 = __fmaf_rn(F6_r11, -0.0530330091714859f, _v100003);
        const float s0_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v100004);
        const float _v100006 = __fmaf_rn(F6_r20, -0.0530330091714859f, F6_t2);
        const float _v100007 = __fmaf_rn(F6_r21, -0.0530330091714859f, _v100006);
        const float s0_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.02800000086426735f);
        const float _v100009 = __fmaf_rn(F6_r00, -0.03181980550289154f, F6_t0);
        const float _v100010 = __fmaf_rn(F6_r01, -0.03181980550289154f, _v100009);
        const float s1_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v100010);
        const float _v100012 = __fmaf_rn(F6_r10, -0.03181980550289154f, F6_t1);
        const float _v100013 = __fmaf_rn(F6_r11, -0.03181980550289154f, _v100012);
        const float s1_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v100013);
        const float _v100015 = __fmaf_rn(F6_r20, -0.03181980550289154f, F6_t2);
        const float _v100016 = __fmaf_rn(F6_r21, -0.03181980550289154f, _v100015);
        const float s1_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.02800000086426735f);
        const float _v100018 = __fmaf_rn(F6_r00, -0.01060660183429718f, F6_t0);
        const float _v100019 = __fmaf_rn(F6_r01, -0.01060660183429718f, _v100018);
        const float s2_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v100019);
        const float _v100021 = __fmaf_rn(F6_r10, -0.01060660183429718f, F6_t1);
        const float _v100022 = __fmaf_rn(F6_r11, -0.01060660183429718f, _v100021);
        const float s2_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v100022);
        const float _v100024 = __fmaf_rn(F6_r20, -0.01060660183429718f, F6_t2);
        const float _v100025 = __fmaf_rn(F6_r21, -0.01060660183429718f, _v100024);
        const float s2_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.02800000086426735f);
        const float _v100027 = __fmaf_rn(F6_r00, 0.01060660183429718f, F6_t0);
        const float _v100028 = __fmaf_rn(F6_r01, 0.01060660183429718f, _v100027);
        const float s3_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v100028);
        const float _v100030 = __fmaf_rn(F6_r10, 0.01060660183429718f, F6_t1);
        const float _v100031 = __fmaf_rn(F6_r11, 0.01060660183429718f, _v100030);
        const float s3_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v100031);
        const float _v100033 = __fmaf_rn(F6_r20, 0.01060660183429718f, F6_t2);
        const float _v100034 = __fmaf_rn(F6_r21, 0.01060660183429718f, _v100033);
        const float s3_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.02800000086426735f);
        const float _v100036 = __fmaf_rn(F6_r00, 0.03181980550289154f, F6_t0);
        const float _v100037 = __fmaf_rn(F6_r01, 0.03181980550289154f, _v100036);
        const float s4_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v100037);
        const float _v100039 = __fmaf_rn(F6_r10, 0.03181980550289154f, F6_t1);
        const float _v100040 = __fmaf_rn(F6_r11, 0.03181980550289154f, _v100039);
        const float s4_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v100040);
        const float _v100042 = __fmaf_rn(F6_r20, 0.03181980550289154f, F6_t2);
        const float _v100043 = __fmaf_rn(F6_r21, 0.03181980550289154f, _v100042);
        const float s4_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v100043);
        out[4] = make_float4(s4_x, s4_y, s4_z, 0.02800000086426735f);
        const float _v100045 = __fmaf_rn(F6_r00, 0.0530330091714859f, F6_t0);
        const float _v100046 = __fmaf_rn(F6_r01, 0.0530330091714859f, _v100045);
        const float s5_x = __fmaf_rn(F6_r02, 0.11699999868869781f, _v100046);
        const float _v100048 = __fmaf_rn(F6_r10, 0.0530330091714859f, F6_t1);
        const float _v100049 = __fmaf_rn(F6_r11, 0.0530330091714859f, _v100048);
        const float s5_y = __fmaf_rn(F6_r12, 0.11699999868869781f, _v100049);
        const float _v100051 = __fmaf_rn(F6_r20, 0.0530330091714859f, F6_t2);
        const float _v100052 = __fmaf_rn(F6_r21, 0.0530330091714859f, _v100051);
        const float s5_z = __fmaf_rn(F6_r22, 0.11699999868869781f, _v100052);
        out[5] = make_float4(s5_x, s5_y, s5_z, 0.02800000086426735f);
        const float _v100054 = __fmaf_rn(F6_r00, -0.0530330091714859f, F6_t0);
        const float _v100055 = __fmaf_rn(F6_r01, -0.0530330091714859f, _v100054);
        const float s6_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v100055);
        const float _v100057 = __fmaf_rn(F6_r10, -0.0530330091714859f, F6_t1);
        const float _v100058 = __fmaf_rn(F6_r11, -0.0530330091714859f, _v100057);
        const float s6_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v100058);
        const float _v100060 = __fmaf_rn(F6_r20, -0.0530330091714859f, F6_t2);
        const float _v100061 = __fmaf_rn(F6_r21, -0.0530330091714859f, _v100060);
        const float s6_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v100061);
        out[6] = make_float4(s6_x, s6_y, s6_z, 0.026000000536441803f);
        const float _v100063 = __fmaf_rn(F6_r00, -0.03181980550289154f, F6_t0);
        const float _v100064 = __fmaf_rn(F6_r01, -0.03181980550289154f, _v100063);
        const float s7_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v100064);
        const float _v100066 = __fmaf_rn(F6_r10, -0.03181980550289154f, F6_t1);
        const float _v100067 = __fmaf_rn(F6_r11, -0.03181980550289154f, _v100066);
        const float s7_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v100067);
        const float _v100069 = __fmaf_rn(F6_r20, -0.03181980550289154f, F6_t2);
        const float _v100070 = __fmaf_rn(F6_r21, -0.03181980550289154f, _v100069);
        const float s7_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v100070);
        out[7] = make_float4(s7_x, s7_y, s7_z, 0.026000000536441803f);
        const float _v100072 = __fmaf_rn(F6_r00, -0.01060660183429718f, F6_t0);
        const float _v100073 = __fmaf_rn(F6_r01, -0.01060660183429718f, _v100072);
        const float s8_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v100073);
        const float _v100075 = __fmaf_rn(F6_r10, -0.01060660183429718f, F6_t1);
        const float _v100076 = __fmaf_rn(F6_r11, -0.01060660183429718f, _v100075);
        const float s8_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v100076);
        const float _v100078 = __fmaf_rn(F6_r20, -0.01060660183429718f, F6_t2);
        const float _v100079 = __fmaf_rn(F6_r21, -0.01060660183429718f, _v100078);
        const float s8_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v100079);
        out[8] = make_float4(s8_x, s8_y, s8_z, 0.026000000536441803f);
        const float _v100081 = __fmaf_rn(F6_r00, 0.01060660183429718f, F6_t0);
        const float _v100082 = __fmaf_rn(F6_r01, 0.01060660183429718f, _v100081);
        const float s9_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v100082);
        const float _v100084 = __fmaf_rn(F6_r10, 0.01060660183429718f, F6_t1);
        const float _v100085 = __fmaf_rn(F6_r11, 0.01060660183429718f, _v100084);
        const float s9_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v100085);
        const float _v100087 = __fmaf_rn(F6_r20, 0.01060660183429718f, F6_t2);
        const float _v100088 = __fmaf_rn(F6_r21, 0.01060660183429718f, _v100087);
        const float s9_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v100088);
        out[9] = make_float4(s9_x, s9_y, s9_z, 0.026000000536441803f);
        const float _v100090 = __fmaf_rn(F6_r00, 0.03181980550289154f, F6_t0);
        const float _v100091 = __fmaf_rn(F6_r01, 0.03181980550289154f, _v100090);
        const float s10_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v100091);
        const float _v100093 = __fmaf_rn(F6_r10, 0.03181980550289154f, F6_t1);
        const float _v100094 = __fmaf_rn(F6_r11, 0.03181980550289154f, _v100093);
        const float s10_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v100094);
        const float _v100096 = __fmaf_rn(F6_r20, 0.03181980550289154f, F6_t2);
        const float _v100097 = __fmaf_rn(F6_r21, 0.03181980550289154f, _v100096);
        const float s10_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v100097);
        out[10] = make_float4(s10_x, s10_y, s10_z, 0.026000000536441803f);
        const float _v100099 = __fmaf_rn(F6_r00, 0.0530330091714859f, F6_t0);
        const float _v100100 = __fmaf_rn(F6_r01, 0.0530330091714859f, _v100099);
        const float s11_x = __fmaf_rn(F6_r02, 0.13699999451637268f, _v100100);
        const float _v100102 = __fmaf_rn(F6_r10, 0.0530330091714859f, F6_t1);
        const float _v100103 = __fmaf_rn(F6_r11, 0.0530330091714859f, _v100102);
        const float s11_y = __fmaf_rn(F6_r12, 0.13699999451637268f, _v100103);
        const float _v100105 = __fmaf_rn(F6_r20, 0.0530330091714859f, F6_t2);
        const float _v100106 = __fmaf_rn(F6_r21, 0.0530330091714859f, _v100105);
        const float s11_z = __fmaf_rn(F6_r22, 0.13699999451637268f, _v100106);
        out[11] = make_float4(s11_x, s11_y, s11_z, 0.026000000536441803f);
        const float _v100108 = __fmaf_rn(F6_r00, -0.0530330091714859f, F6_t0);
        const float _v100109 = __fmaf_rn(F6_r01, -0.0530330091714859f, _v100108);
        const float s12_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v100109);
        const float _v100111 = __fmaf_rn(F6_r10, -0.0530330091714859f, F6_t1);
        const float _v100112 = __fmaf_rn(F6_r11, -0.0530330091714859f, _v100111);
        const float s12_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v100112);
        const float _v100114 = __fmaf_rn(F6_r20, -0.0530330091714859f, F6_t2);
        const float _v100115 = __fmaf_rn(F6_r21, -0.0530330091714859f, _v100114);
        const float s12_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v100115);
        out[12] = make_float4(s12_x, s12_y, s12_z, 0.024000000208616257f);
        const float _v100117 = __fmaf_rn(F6_r00, -0.03181980550289154f, F6_t0);
        const float _v100118 = __fmaf_rn(F6_r01, -0.03181980550289154f, _v100117);
        const float s13_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v100118);
        const float _v100120 = __fmaf_rn(F6_r10, -0.03181980550289154f, F6_t1);
        const float _v100121 = __fmaf_rn(F6_r11, -0.03181980550289154f, _v100120);
        const float s13_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v100121);
        const float _v100123 = __fmaf_rn(F6_r20, -0.03181980550289154f, F6_t2);
        const float _v100124 = __fmaf_rn(F6_r21, -0.03181980550289154f, _v100123);
        const float s13_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v100124);
        out[13] = make_float4(s13_x, s13_y, s13_z, 0.024000000208616257f);
        const float _v100126 = __fmaf_rn(F6_r00, -0.01060660183429718f, F6_t0);
        const float _v100127 = __fmaf_rn(F6_r01, -0.01060660183429718f, _v100126);
        const float s14_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v100127);
        const float _v100129 = __fmaf_rn(F6_r10, -0.01060660183429718f, F6_t1);
        const float _v100130 = __fmaf_rn(F6_r11, -0.01060660183429718f, _v100129);
        const float s14_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v100130);
        const float _v100132 = __fmaf_rn(F6_r20, -0.01060660183429718f, F6_t2);
        const float _v100133 = __fmaf_rn(F6_r21, -0.01060660183429718f, _v100132);
        const float s14_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v100133);
        out[14] = make_float4(s14_x, s14_y, s14_z, 0.024000000208616257f);
        const float _v100135 = __fmaf_rn(F6_r00, 0.01060660183429718f, F6_t0);
        const float _v100136 = __fmaf_rn(F6_r01, 0.01060660183429718f, _v100135);
        const float s15_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v100136);
        const float _v100138 = __fmaf_rn(F6_r10, 0.01060660183429718f, F6_t1);
        const float _v100139 = __fmaf_rn(F6_r11, 0.01060660183429718f, _v100138);
        const float s15_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v100139);
        const float _v100141 = __fmaf_rn(F6_r20, 0.01060660183429718f, F6_t2);
        const float _v100142 = __fmaf_rn(F6_r21, 0.01060660183429718f, _v100141);
        const float s15_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v100142);
        out[15] = make_float4(s15_x, s15_y, s15_z, 0.024000000208616257f);
        const float _v100144 = __fmaf_rn(F6_r00, 0.03181980550289154f, F6_t0);
        const float _v100145 = __fmaf_rn(F6_r01, 0.03181980550289154f, _v100144);
        const float s16_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v100145);
        const float _v100147 = __fmaf_rn(F6_r10, 0.03181980550289154f, F6_t1);
        const float _v100148 = __fmaf_rn(F6_r11, 0.03181980550289154f, _v100147);
        const float s16_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v100148);
        const float _v100150 = __fmaf_rn(F6_r20, 0.03181980550289154f, F6_t2);
        const float _v100151 = __fmaf_rn(F6_r21, 0.03181980550289154f, _v100150);
        const float s16_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v100151);
        out[16] = make_float4(s16_x, s16_y, s16_z, 0.024000000208616257f);
        const float _v100153 = __fmaf_rn(F6_r00, 0.0530330091714859f, F6_t0);
        const float _v100154 = __fmaf_rn(F6_r01, 0.0530330091714859f, _v100153);
        const float s17_x = __fmaf_rn(F6_r02, 0.15700000524520874f, _v100154);
        const float _v100156 = __fmaf_rn(F6_r10, 0.0530330091714859f, F6_t1);
        const float _v100157 = __fmaf_rn(F6_r11, 0.0530330091714859f, _v100156);
        const float s17_y = __fmaf_rn(F6_r12, 0.15700000524520874f, _v100157);
        const float _v100159 = __fmaf_rn(F6_r20, 0.0530330091714859f, F6_t2);
        const float _v100160 = __fmaf_rn(F6_r21, 0.0530330091714859f, _v100159);
        const float s17_z = __fmaf_rn(F6_r22, 0.15700000524520874f, _v100160);
        out[17] = make_float4(s17_x, s17_y, s17_z, 0.024000000208616257f);
    }
    // fine spheres [32, 33, 34, 35, 36] (panda_link7)
    static __device__ __noinline__ void fine_3(const float F6_r00, const float F6_r01, const float F6_r02, const float F6_r10, const float F6_r11, const float F6_r12, const float F6_r20, const float F6_r21, const float F6_r22, const float F6_t0, const float F6_t1, const float F6_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
        const float _v100001 = __fmaf_rn(F6_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(F6_r02, 0.07000000029802322f, _v100001);
        const float _v100003 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
        const float _v100004 = __fmaf_rn(F6_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(F6_r12, 0.07000000029802322f, _v100004);
        const float _v100006 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
        const float _v100007 = __fmaf_rn(F6_r21, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(F6_r22, 0.07000000029802322f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05000000074505806f);
        const float _v100009 = __fmaf_rn(F6_r00, 0.019999999552965164f, F6_t0);
        const float _v100010 = __fmaf_rn(F6_r01, 0.03999999910593033f, _v100009);
        const float s1_x = __fmaf_rn(F6_r02, 0.07999999821186066f, _v100010);
        const float _v100012 = __fmaf_rn(F6_r10, 0.019999999552965164f, F6_t1);
        const float _v100013 = __fmaf_rn(F6_r11, 0.03999999910593033f, _v100012);
        const float s1_y = __fmaf_rn(F6_r12, 0.07999999821186066f, _v100013);
        const float _v100015 = __fmaf_rn(F6_r20, 0.019999999552965164f, F6_t2);
        const float _v100016 = __fmaf_rn(F6_r21, 0.03999999910593033f, _v100015);
        const float s1_z = __fmaf_rn(F6_r22, 0.07999999821186066f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.02500000037252903f);
        const float _v100018 = __fmaf_rn(F6_r00, 0.03999999910593033f, F6_t0);
        const float _v100019 = __fmaf_rn(F6_r01, 0.019999999552965164f, _v100018);
        const float s2_x = __fmaf_rn(F6_r02, 0.07999999821186066f, _v100019);
        const float _v100021 = __fmaf_rn(F6_r10, 0.03999999910593033f, F6_t1);
        const float _v100022 = __fmaf_rn(F6_r11, 0.019999999552965164f, _v100021);
        const float s2_y = __fmaf_rn(F6_r12, 0.07999999821186066f, _v100022);
        const float _v100024 = __fmaf_rn(F6_r20, 0.03999999910593033f, F6_t2);
        const float _v100025 = __fmaf_rn(F6_r21, 0.019999999552965164f, _v100024);
        const float s2_z = __fmaf_rn(F6_r22, 0.07999999821186066f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.02500000037252903f);
        const float _v100027 = __fmaf_rn(F6_r00, 0.03999999910593033f, F6_t0);
        const float _v100028 = __fmaf_rn(F6_r01, 0.05999999865889549f, _v100027);
        const float s3_x = __fmaf_rn(F6_r02, 0.08500000089406967f, _v100028);
        const float _v100030 = __fmaf_rn(F6_r10, 0.03999999910593033f, F6_t1);
        const float _v100031 = __fmaf_rn(F6_r11, 0.05999999865889549f, _v100030);
        const float s3_y = __fmaf_rn(F6_r12, 0.08500000089406967f, _v100031);
        const float _v100033 = __fmaf_rn(F6_r20, 0.03999999910593033f, F6_t2);
        const float _v100034 = __fmaf_rn(F6_r21, 0.05999999865889549f, _v100033);
        const float s3_z = __fmaf_rn(F6_r22, 0.08500000089406967f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.019999999552965164f);
        const float _v100036 = __fmaf_rn(F6_r00, 0.05999999865889549f, F6_t0);
        const float _v100037 = __fmaf_rn(F6_r01, 0.03999999910593033f, _v100036);
        const float s4_x = __fmaf_rn(F6_r02, 0.08500000089406967f, _v100037);
        const float _v100039 = __fmaf_rn(F6_r10, 0.05999999865889549f, F6_t1);
        const float _v100040 = __fmaf_rn(F6_r11, 0.03999999910593033f, _v100039);
        const float s4_y = __fmaf_rn(F6_r12, 0.08500000089406967f, _v100040);
        const float _v100042 = __fmaf_rn(F6_r20, 0.05999999865889549f, F6_t2);
        const float _v100043 = __fmaf_rn(F6_r21, 0.03999999910593033f, _v100042);
        const float s4_z = __fmaf_rn(F6_r22, 0.08500000089406967f, _v100043);
        out[4] = make_float4(s4_x, s4_y, s4_z, 0.019999999552965164f);
    }
    // fine spheres [29, 30, 31] (panda_link6)
    static __device__ __noinline__ void fine_4(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05000000074505806f);
        const float _v100009 = __fmaf_rn(F5_r00, 0.07999999821186066f, F5_t0);
        const float _v100010 = __fmaf_rn(F5_r01, -0.009999999776482582f, _v100009);
        const float s1_x = __fmaf_rn(F5_r02, 0.0f, _v100010);
        const float _v100012 = __fmaf_rn(F5_r10, 0.07999999821186066f, F5_t1);
        const float _v100013 = __fmaf_rn(F5_r11, -0.009999999776482582f, _v100012);
        const float s1_y = __fmaf_rn(F5_r12, 0.0f, _v100013);
        const float _v100015 = __fmaf_rn(F5_r20, 0.07999999821186066f, F5_t2);
        const float _v100016 = __fmaf_rn(F5_r21, -0.009999999776482582f, _v100015);
        const float s1_z = __fmaf_rn(F5_r22, 0.0f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.05000000074505806f);
        const float _v100018 = __fmaf_rn(F5_r00, 0.07999999821186066f, F5_t0);
        const float _v100019 = __fmaf_rn(F5_r01, 0.03500000014901161f, _v100018);
        const float s2_x = __fmaf_rn(F5_r02, 0.0f, _v100019);
        const float _v100021 = __fmaf_rn(F5_r10, 0.07999999821186066f, F5_t1);
        const float _v100022 = __fmaf_rn(F5_r11, 0.03500000014901161f, _v100021);
        const float s2_y = __fmaf_rn(F5_r12, 0.0f, _v100022);
        const float _v100024 = __fmaf_rn(F5_r20, 0.07999999821186066f, F5_t2);
        const float _v100025 = __fmaf_rn(F5_r21, 0.03500000014901161f, _v100024);
        const float s2_z = __fmaf_rn(F5_r22, 0.0f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.052000001072883606f);
    }
    // fine spheres [17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28] (panda_link5)
    static __device__ __noinline__ void fine_5(const float F4_r00, const float F4_r01, const float F4_r02, const float F4_r10, const float F4_r11, const float F4_r12, const float F4_r20, const float F4_r21, const float F4_r22, const float F4_t0, const float F4_t1, const float F4_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100001 = __fmaf_rn(F4_r01, 0.054999999701976776f, _v100000);
        const float s0_x = __fmaf_rn(F4_r02, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100004 = __fmaf_rn(F4_r11, 0.054999999701976776f, _v100003);
        const float s0_y = __fmaf_rn(F4_r12, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100007 = __fmaf_rn(F4_r21, 0.054999999701976776f, _v100006);
        const float s0_z = __fmaf_rn(F4_r22, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05999999865889549f);
        const float _v100009 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100010 = __fmaf_rn(F4_r01, 0.07500000298023224f, _v100009);
        const float s1_x = __fmaf_rn(F4_r02, 0.0f, _v100010);
        const float _v100012 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100013 = __fmaf_rn(F4_r11, 0.07500000298023224f, _v100012);
        const float s1_y = __fmaf_rn(F4_r12, 0.0f, _v100013);
        const float _v100015 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100016 = __fmaf_rn(F4_r21, 0.07500000298023224f, _v100015);
        const float s1_z = __fmaf_rn(F4_r22, 0.0f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.05999999865889549f);
        const float _v100018 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100019 = __fmaf_rn(F4_r01, 0.0f, _v100018);
        const float s2_x = __fmaf_rn(F4_r02, -0.2199999988079071f, _v100019);
        const float _v100021 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100022 = __fmaf_rn(F4_r11, 0.0f, _v100021);
        const float s2_y = __fmaf_rn(F4_r12, -0.2199999988079071f, _v100022);
        const float _v100024 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100025 = __fmaf_rn(F4_r21, 0.0f, _v100024);
        const float s2_z = __fmaf_rn(F4_r22, -0.2199999988079071f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.05999999865889549f);
        const float _v100027 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100028 = __fmaf_rn(F4_r01, 0.05000000074505806f, _v100027);
        const float s3_x = __fmaf_rn(F4_r02, -0.18000000715255737f, _v100028);
        const float _v100030 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100031 = __fmaf_rn(F4_r11, 0.05000000074505806f, _v100030);
        const float s3_y = __fmaf_rn(F4_r12, -0.18000000715255737f, _v100031);
        const float _v100033 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100034 = __fmaf_rn(F4_r21, 0.05000000074505806f, _v100033);
        const float s3_z = __fmaf_rn(F4_r22, -0.18000000715255737f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.05000000074505806f);
        const float _v100036 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v100037 = __fmaf_rn(F4_r01, 0.07999999821186066f, _v100036);
        const float s4_x = __fmaf_rn(F4_r02, -0.14000000059604645f, _v100037);
        const float _v100039 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v100040 = __fmaf_rn(F4_r11, 0.07999999821186066f, _v100039);
        const float s4_y = __fmaf_rn(F4_r12, -0.14000000059604645f, _v100040);
        const float _v100042 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v100043 = __fmaf_rn(F4_r21, 0.07999999821186066f, _v100042);
        const float s4_z = __fmaf_rn(F4_r22, -0.14000000059604645f, _v100043);
        out[4] = make_float4(s4_x, s4_y, s4_z, 0.02500000037252903f);
        const float _v100045 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v100046 = __fmaf_rn(F4_r01, 0.08500000089406967f, _v100045);
        const float s5_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v100046);
        const float _v100048 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v100049 = __fmaf_rn(F4_r11, 0.08500000089406967f, _v100048);
        const float s5_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v100049);
        const float _v100051 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v100052 = __fmaf_rn(F4_r21, 0.08500000089406967f, _v100051);
        const float s5_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v100052);
        out[5] = make_float4(s5_x, s5_y, s5_z, 0.02500000037252903f);
        const float _v100054 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v100055 = __fmaf_rn(F4_r01, 0.09000000357627869f, _v100054);
        const float s6_x = __fmaf_rn(F4_r02, -0.07999999821186066f, _v100055);
        const float _v100057 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v100058 = __fmaf_rn(F4_r11, 0.09000000357627869f, _v100057);
        const float s6_y = __fmaf_rn(F4_r12, -0.07999999821186066f, _v100058);
        const float _v100060 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v100061 = __fmaf_rn(F4_r21, 0.09000000357627869f, _v100060);
        const float s6_z = __fmaf_rn(F4_r22, -0.07999999821186066f, _v100061);
        out[6] = make_float4(s6_x, s6_y, s6_z, 0.02500000037252903f);
        const float _v100063 = __fmaf_rn(F4_r00, 0.009999999776482582f, F4_t0);
        const float _v100064 = __fmaf_rn(F4_r01, 0.0949999988079071f, _v100063);
        const float s7_x = __fmaf_rn(F4_r02, -0.05000000074505806f, _v100064);
        const float _v100066 = __fmaf_rn(F4_r10, 0.009999999776482582f, F4_t1);
        const float _v100067 = __fmaf_rn(F4_r11, 0.0949999988079071f, _v100066);
        const float s7_y = __fmaf_rn(F4_r12, -0.05000000074505806f, _v100067);
        const float _v100069 = __fmaf_rn(F4_r20, 0.009999999776482582f, F4_t2);
        const float _v100070 = __fmaf_rn(F4_r21, 0.0949999988079071f, _v100069);
        const float s7_z = __fmaf_rn(F4_r22, -0.05000000074505806f, _v100070);
        out[7] = make_float4(s7_x, s7_y, s7_z, 0.02500000037252903f);
        const float _v100072 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v100073 = __fmaf_rn(F4_r01, 0.07999999821186066f, _v100072);
        const float s8_x = __fmaf_rn(F4_r02, -0.14000000059604645f, _v100073);
        const float _v100075 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v100076 = __fmaf_rn(F4_r11, 0.07999999821186066f, _v100075);
        const float s8_y = __fmaf_rn(F4_r12, -0.14000000059604645f, _v100076);
        const float _v100078 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v100079 = __fmaf_rn(F4_r21, 0.07999999821186066f, _v100078);
        const float s8_z = __fmaf_rn(F4_r22, -0.14000000059604645f, _v100079);
        out[8] = make_float4(s8_x, s8_y, s8_z, 0.02500000037252903f);
        const float _v100081 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v100082 = __fmaf_rn(F4_r01, 0.08500000089406967f, _v100081);
        const float s9_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v100082);
        const float _v100084 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v100085 = __fmaf_rn(F4_r11, 0.08500000089406967f, _v100084);
        const float s9_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v100085);
        const float _v100087 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v100088 = __fmaf_rn(F4_r21, 0.08500000089406967f, _v100087);
        const float s9_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v100088);
        out[9] = make_float4(s9_x, s9_y, s9_z, 0.02500000037252903f);
        const float _v100090 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v100091 = __fmaf_rn(F4_r01, 0.09000000357627869f, _v100090);
        const float s10_x = __fmaf_rn(F4_r02, -0.07999999821186066f, _v100091);
        const float _v100093 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v100094 = __fmaf_rn(F4_r11, 0.09000000357627869f, _v100093);
        const float s10_y = __fmaf_rn(F4_r12, -0.07999999821186066f, _v100094);
        const float _v100096 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v100097 = __fmaf_rn(F4_r21, 0.09000000357627869f, _v100096);
        const float s10_z = __fmaf_rn(F4_r22, -0.07999999821186066f, _v100097);
        out[10] = make_float4(s10_x, s10_y, s10_z, 0.02500000037252903f);
        const float _v100099 = __fmaf_rn(F4_r00, -0.009999999776482582f, F4_t0);
        const float _v100100 = __fmaf_rn(F4_r01, 0.0949999988079071f, _v100099);
        const float s11_x = __fmaf_rn(F4_r02, -0.05000000074505806f, _v100100);
        const float _v100102 = __fmaf_rn(F4_r10, -0.009999999776482582f, F4_t1);
        const float _v100103 = __fmaf_rn(F4_r11, 0.0949999988079071f, _v100102);
        const float s11_y = __fmaf_rn(F4_r12, -0.05000000074505806f, _v100103);
        const float _v100105 = __fmaf_rn(F4_r20, -0.009999999776482582f, F4_t2);
        const float _v100106 = __fmaf_rn(F4_r21, 0.0949999988079071f, _v100105);
        const float s11_z = __fmaf_rn(F4_r22, -0.05000000074505806f, _v100106);
        out[11] = make_float4(s11_x, s11_y, s11_z, 0.02500000037252903f);
    }
    // fine spheres [13, 14, 15, 16] (panda_link4)
    static __device__ __noinline__ void fine_6(const float F3_r00, const float F3_r01, const float F3_r02, const float F3_r10, const float F3_r11, const float F3_r12, const float F3_r20, const float F3_r21, const float F3_r22, const float F3_t0, const float F3_t1, const float F3_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F3_r00, -0.07999999821186066f, F3_t0);
        const float _v100001 = __fmaf_rn(F3_r01, 0.0949999988079071f, _v100000);
        const float s0_x = __fmaf_rn(F3_r02, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F3_r10, -0.07999999821186066f, F3_t1);
        const float _v100004 = __fmaf_rn(F3_r11, 0.0949999988079071f, _v100003);
        const float s0_y = __fmaf_rn(F3_r12, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(F3_r20, -0.07999999821186066f, F3_t2);
        const float _v100007 = __fmaf_rn(F3_r21, 0.0949999988079071f, _v100006);
        const float s0_z = __fmaf_rn(F3_r22, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05999999865889549f);
        const float _v100009 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v100010 = __fmaf_rn(F3_r01, 0.0f, _v100009);
        const float s1_x = __fmaf_rn(F3_r02, 0.019999999552965164f, _v100010);
        const float _v100012 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v100013 = __fmaf_rn(F3_r11, 0.0f, _v100012);
        const float s1_y = __fmaf_rn(F3_r12, 0.019999999552965164f, _v100013);
        const float _v100015 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v100016 = __fmaf_rn(F3_r21, 0.0f, _v100015);
        const float s1_z = __fmaf_rn(F3_r22, 0.019999999552965164f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.054999999701976776f);
        const float _v100018 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v100019 = __fmaf_rn(F3_r01, 0.0f, _v100018);
        const float s2_x = __fmaf_rn(F3_r02, 0.05999999865889549f, _v100019);
        const float _v100021 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v100022 = __fmaf_rn(F3_r11, 0.0f, _v100021);
        const float s2_y = __fmaf_rn(F3_r12, 0.05999999865889549f, _v100022);
        const float _v100024 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v100025 = __fmaf_rn(F3_r21, 0.0f, _v100024);
        const float s2_z = __fmaf_rn(F3_r22, 0.05999999865889549f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.054999999701976776f);
        const float _v100027 = __fmaf_rn(F3_r00, -0.07999999821186066f, F3_t0);
        const float _v100028 = __fmaf_rn(F3_r01, 0.05999999865889549f, _v100027);
        const float s3_x = __fmaf_rn(F3_r02, 0.0f, _v100028);
        const float _v100030 = __fmaf_rn(F3_r10, -0.07999999821186066f, F3_t1);
        const float _v100031 = __fmaf_rn(F3_r11, 0.05999999865889549f, _v100030);
        const float s3_y = __fmaf_rn(F3_r12, 0.0f, _v100031);
        const float _v100033 = __fmaf_rn(F3_r20, -0.07999999821186066f, F3_t2);
        const float _v100034 = __fmaf_rn(F3_r21, 0.05999999865889549f, _v100033);
        const float s3_z = __fmaf_rn(F3_r22, 0.0f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.054999999701976776f);
    }
    // fine spheres [9, 10, 11, 12] (panda_link3)
    static __device__ __noinline__ void fine_7(const float F2_r00, const float F2_r01, const float F2_r02, const float F2_r10, const float F2_r11, const float F2_r12, const float F2_r20, const float F2_r21, const float F2_r22, const float F2_t0, const float F2_t1, const float F2_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100001 = __fmaf_rn(F2_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(F2_r02, -0.10000000149011612f, _v100001);
        const float _v100003 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100004 = __fmaf_rn(F2_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(F2_r12, -0.10000000149011612f, _v100004);
        const float _v100006 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100007 = __fmaf_rn(F2_r21, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(F2_r22, -0.10000000149011612f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05999999865889549f);
        const float _v100009 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100010 = __fmaf_rn(F2_r01, 0.0f, _v100009);
        const float s1_x = __fmaf_rn(F2_r02, -0.05999999865889549f, _v100010);
        const float _v100012 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100013 = __fmaf_rn(F2_r11, 0.0f, _v100012);
        const float s1_y = __fmaf_rn(F2_r12, -0.05999999865889549f, _v100013);
        const float _v100015 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100016 = __fmaf_rn(F2_r21, 0.0f, _v100015);
        const float s1_z = __fmaf_rn(F2_r22, -0.05999999865889549f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.05000000074505806f);
        const float _v100018 = __fmaf_rn(F2_r00, 0.07999999821186066f, F2_t0);
        const float _v100019 = __fmaf_rn(F2_r01, 0.05999999865889549f, _v100018);
        const float s2_x = __fmaf_rn(F2_r02, 0.0f, _v100019);
        const float _v100021 = __fmaf_rn(F2_r10, 0.07999999821186066f, F2_t1);
        const float _v100022 = __fmaf_rn(F2_r11, 0.05999999865889549f, _v100021);
        const float s2_y = __fmaf_rn(F2_r12, 0.0f, _v100022);
        const float _v100024 = __fmaf_rn(F2_r20, 0.07999999821186066f, F2_t2);
        const float _v100025 = __fmaf_rn(F2_r21, 0.05999999865889549f, _v100024);
        const float s2_z = __fmaf_rn(F2_r22, 0.0f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.054999999701976776f);
        const float _v100027 = __fmaf_rn(F2_r00, 0.07999999821186066f, F2_t0);
        const float _v100028 = __fmaf_rn(F2_r01, 0.019999999552965164f, _v100027);
        const float s3_x = __fmaf_rn(F2_r02, 0.0f, _v100028);
        const float _v100030 = __fmaf_rn(F2_r10, 0.07999999821186066f, F2_t1);
        const float _v100031 = __fmaf_rn(F2_r11, 0.019999999552965164f, _v100030);
        const float s3_y = __fmaf_rn(F2_r12, 0.0f, _v100031);
        const float _v100033 = __fmaf_rn(F2_r20, 0.07999999821186066f, F2_t2);
        const float _v100034 = __fmaf_rn(F2_r21, 0.019999999552965164f, _v100033);
        const float s3_z = __fmaf_rn(F2_r22, 0.0f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.054999999701976776f);
    }
    // fine spheres [5, 6, 7, 8] (panda_link2)
    static __device__ __noinline__ void fine_8(const float F1_r00, const float F1_r01, const float F1_r02, const float F1_r10, const float F1_r11, const float F1_r12, const float F1_r20, const float F1_r21, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v100001 = __fmaf_rn(F1_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(F1_r02, 0.029999999329447746f, _v100001);
        const float _v100003 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v100004 = __fmaf_rn(F1_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(F1_r12, 0.029999999329447746f, _v100004);
        const float _v100006 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v100007 = __fmaf_rn(F1_r21, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(0.0f, 0.029999999329447746f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05999999865889549f);
        const float _v100009 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v100010 = __fmaf_rn(F1_r01, 0.0f, _v100009);
        const float s1_x = __fmaf_rn(F1_r02, 0.07999999821186066f, _v100010);
        const float _v100012 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v100013 = __fmaf_rn(F1_r11, 0.0f, _v100012);
        const float s1_y = __fmaf_rn(F1_r12, 0.07999999821186066f, _v100013);
        const float _v100015 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v100016 = __fmaf_rn(F1_r21, 0.0f, _v100015);
        const float s1_z = __fmaf_rn(0.0f, 0.07999999821186066f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.05999999865889549f);
        const float _v100018 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v100019 = __fmaf_rn(F1_r01, -0.11999999731779099f, _v100018);
        const float s2_x = __fmaf_rn(F1_r02, 0.0f, _v100019);
        const float _v100021 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v100022 = __fmaf_rn(F1_r11, -0.11999999731779099f, _v100021);
        const float s2_y = __fmaf_rn(F1_r12, 0.0f, _v100022);
        const float _v100024 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v100025 = __fmaf_rn(F1_r21, -0.11999999731779099f, _v100024);
        const float s2_z = __fmaf_rn(0.0f, 0.0f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.05999999865889549f);
        const float _v100027 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
        const float _v100028 = __fmaf_rn(F1_r01, -0.17000000178813934f, _v100027);
        const float s3_x = __fmaf_rn(F1_r02, 0.0f, _v100028);
        const float _v100030 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
        const float _v100031 = __fmaf_rn(F1_r11, -0.17000000178813934f, _v100030);
        const float s3_y = __fmaf_rn(F1_r12, 0.0f, _v100031);
        const float _v100033 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
        const float _v100034 = __fmaf_rn(F1_r21, -0.17000000178813934f, _v100033);
        const float s3_z = __fmaf_rn(0.0f, 0.0f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.05999999865889549f);
    }
    // fine spheres [1, 2, 3, 4] (panda_link1)
    static __device__ __noinline__ void fine_9(const float F0_r00, const float F0_r01, const float F0_r10, const float F0_r11, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v100001 = __fmaf_rn(F0_r01, -0.07999999821186066f, _v100000);
        const float s0_x = __fmaf_rn(0.0f, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v100004 = __fmaf_rn(F0_r11, -0.07999999821186066f, _v100003);
        const float s0_y = __fmaf_rn(0.0f, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v100007 = __fmaf_rn(0.0f, -0.07999999821186066f, _v100006);
        const float s0_z = __fmaf_rn(1.0f, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.05999999865889549f);
        const float _v100009 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v100010 = __fmaf_rn(F0_r01, -0.029999999329447746f, _v100009);
        const float s1_x = __fmaf_rn(0.0f, 0.0f, _v100010);
        const float _v100012 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v100013 = __fmaf_rn(F0_r11, -0.029999999329447746f, _v100012);
        const float s1_y = __fmaf_rn(0.0f, 0.0f, _v100013);
        const float _v100015 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v100016 = __fmaf_rn(0.0f, -0.029999999329447746f, _v100015);
        const float s1_z = __fmaf_rn(1.0f, 0.0f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.05999999865889549f);
        const float _v100018 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v100019 = __fmaf_rn(F0_r01, 0.0f, _v100018);
        const float s2_x = __fmaf_rn(0.0f, -0.11999999731779099f, _v100019);
        const float _v100021 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v100022 = __fmaf_rn(F0_r11, 0.0f, _v100021);
        const float s2_y = __fmaf_rn(0.0f, -0.11999999731779099f, _v100022);
        const float _v100024 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v100025 = __fmaf_rn(0.0f, 0.0f, _v100024);
        const float s2_z = __fmaf_rn(1.0f, -0.11999999731779099f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.05999999865889549f);
        const float _v100027 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v100028 = __fmaf_rn(F0_r01, 0.0f, _v100027);
        const float s3_x = __fmaf_rn(0.0f, -0.17000000178813934f, _v100028);
        const float _v100030 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v100031 = __fmaf_rn(F0_r11, 0.0f, _v100030);
        const float s3_y = __fmaf_rn(0.0f, -0.17000000178813934f, _v100031);
        const float _v100033 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
        const float _v100034 = __fmaf_rn(0.0f, 0.0f, _v100033);
        const float s3_z = __fmaf_rn(1.0f, -0.17000000178813934f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.05999999865889549f);
    }
    // fine spheres [0] (panda_link0)
    static __device__ __noinline__ void fine_10(float4 *out)
    {
        const float _v100000 = __fmaf_rn(1.0f, 0.0f, 0.0f);
        const float _v100001 = __fmaf_rn(0.0f, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v100001);
        const float _v100003 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v100004 = __fmaf_rn(1.0f, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v100004);
        const float _v100006 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v100007 = __fmaf_rn(0.0f, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.07999999821186066f);
    }

    // Robot::fkcc for the lanes of ctx.alive.  Clears the lanes of every segment found in collision.
    template <typename Ctx>
    static __device__ __forceinline__ void fkcc(const float *q, Ctx &ctx)
    {
        float F0_s, F0_c; vg_sincos_ref(q[0], &F0_s, &F0_c);
        const float F0_r00 = F0_c;
        const float F0_r01 = (-F0_s);
        const float F0_r10 = F0_s;
        const float F0_r11 = F0_c;
        float F1_s, F1_c; vg_sincos_ref(q[1], &F1_s, &F1_c);
        const float F1_r00 = __fmul_rn(F0_r00, F1_c);
        const float F1_r01 = __fmul_rn((-F0_r00), F1_s);
        const float F1_r02 = F0_r01;
        const float F1_r10 = __fmul_rn(F0_r10, F1_c);
        const float F1_r11 = __fmul_rn((-F0_r10), F1_s);
        const float F1_r12 = F0_r11;
        const float F1_r20 = (-F1_s);
        const float F1_r21 = (-F1_c);
        const float _v4 = __fmul_rn(-0.3160000145435333f, F1_r01);
        const float _v5 = __fmul_rn(-0.3160000145435333f, F1_r11);
        const float _v6 = __fmaf_rn(-0.3160000145435333f, F1_r21, 0.3330000042915344f);
        float F2_s, F2_c; vg_sincos_ref(q[2], &F2_s, &F2_c);
        const float _v7 = __fmul_rn(F1_r00, F2_c);
        const float F2_r00 = __fmaf_rn(F1_r02, F2_s, _v7);
        const float _v9 = __fmul_rn((-F1_r00), F2_s);
        const float F2_r01 = __fmaf_rn(F1_r02, F2_c, _v9);
        const float F2_r02 = (-F1_r01);
        const float _v11 = __fmul_rn(F1_r10, F2_c);
        const float F2_r10 = __fmaf_rn(F1_r12, F2_s, _v11);
        const float _v13 = __fmul_rn((-F1_r10), F2_s);
        const float F2_r11 = __fmaf_rn(F1_r12, F2_c, _v13);
        const float F2_r12 = (-F1_r11);
        const float F2_r20 = __fmul_rn(F1_r20, F2_c);
        const float F2_r21 = __fmul_rn((-F1_r20), F2_s);
        const float F2_r22 = (-F1_r21);
        const float F2_t0 = _v4;
        const float F2_t1 = _v5;
        const float F2_t2 = _v6;
        const float _v17 = __fmaf_rn(0.08250000327825546f, F2_r00, F2_t0);
        const float _v18 = __fmaf_rn(0.08250000327825546f, F2_r10, F2_t1);
        const float _v19 = __fmaf_rn(0.08250000327825546f, F2_r20, F2_t2);
        float F3_s, F3_c; vg_sincos_ref(q[3], &F3_s, &F3_c);
        const float _v20 = __fmul_rn(F2_r00, F3_c);
        const float F3_r00 = __fmaf_rn(F2_r02, F3_s, _v20);
        const float _v22 = __fmul_rn((-F2_r00), F3_s);
        const float F3_r01 = __fmaf_rn(F2_r02, F3_c, _v22);
        const float F3_r02 = (-F2_r01);
        const float _v24 = __fmul_rn(F2_r10, F3_c);
        const float F3_r10 = __fmaf_rn(F2_r12, F3_s, _v24);
        const float _v26 = __fmul_rn((-F2_r10), F3_s);
        const float F3_r11 = __fmaf_rn(F2_r12, F3_c, _v26);
        const float F3_r12 = (-F2_r11);
        const float _v28 = __fmul_rn(F2_r20, F3_c);
        const float F3_r20 = __fmaf_rn(F2_r22, F3_s, _v28);
        const float _v30 = __fmul_rn((-F2_r20), F3_s);
        const float F3_r21 = __fmaf_rn(F2_r22, F3_c, _v30);
        const float F3_r22 = (-F2_r21);
        const float F3_t0 = _v17;
        const float F3_t1 = _v18;
        const float F3_t2 = _v19;
        const float _v32 = __fmaf_rn(-0.08250000327825546f, F3_r00, F3_t0);
        const float _v33 = __fmaf_rn(0.3840000033378601f, F3_r01, _v32);
        const float _v34 = __fmaf_rn(-0.08250000327825546f, F3_r10, F3_t1);
        const float _v35 = __fmaf_rn(0.3840000033378601f, F3_r11, _v34);
        const float _v36 = __fmaf_rn(-0.08250000327825546f, F3_r20, F3_t2);
        const float _v37 = __fmaf_rn(0.3840000033378601f, F3_r21, _v36);
        float F4_s, F4_c; vg_sincos_ref(q[4], &F4_s, &F4_c);
        const float _v38 = __fmul_rn(F3_r00, F4_c);
        const float F4_r00 = __fmaf_rn((-F3_r02), F4_s, _v38);
        const float _v40 = __fmul_rn((-F3_r00), F4_s);
        const float F4_r01 = __fmaf_rn((-F3_r02), F4_c, _v40);
        const float F4_r02 = F3_r01;
        const float _v42 = __fmul_rn(F3_r10, F4_c);
        const float F4_r10 = __fmaf_rn((-F3_r12), F4_s, _v42);
        const float _v44 = __fmul_rn((-F3_r10), F4_s);
        const float F4_r11 = __fmaf_rn((-F3_r12), F4_c, _v44);
        const float F4_r12 = F3_r11;
        const float _v46 = __fmul_rn(F3_r20, F4_c);
        const float F4_r20 = __fmaf_rn((-F3_r22), F4_s, _v46);
        const float _v48 = __fmul_rn((-F3_r20), F4_s);
        const float F4_r21 = __fmaf_rn((-F3_r22), F4_c, _v48);
        const float F4_r22 = F3_r21;
        const float F4_t0 = _v33;
        const float F4_t1 = _v35;
        const float F4_t2 = _v37;
        float F5_s, F5_c; vg_sincos_ref(q[5], &F5_s, &F5_c);
        const float _v50 = __fmul_rn(F4_r00, F5_c);
        const float F5_r00 = __fmaf_rn(F4_r02, F5_s, _v50);
        const float _v52 = __fmul_rn((-F4_r00), F5_s);
        const float F5_r01 = __fmaf_rn(F4_r02, F5_c, _v52);
        const float F5_r02 = (-F4_r01);
        const float _v54 = __fmul_rn(F4_r10, F5_c);
        const float F5_r10 = __fmaf_rn(F4_r12, F5_s, _v54);
        const float _v56 = __fmul_rn((-F4_r10), F5_s);
        const float F5_r11 = __fmaf_rn(F4_r12, F5_c, _v56);
        const float F5_r12 = (-F4_r11);
        const float _v58 = __fmul_rn(F4_r20, F5_c);
        const float F5_r20 = __fmaf_rn(F4_r22, F5_s, _v58);
        const float _v60 = __fmul_rn((-F4_r20), F5_s);
        const float F5_r21 = __fmaf_rn(F4_r22, F5_c, _v60);
        const float F5_r22 = (-F4_r21);
        const float F5_t0 = F4_t0;
        const float F5_t1 = F4_t1;
        const float F5_t2 = F4_t2;
        const float _v62 = __fmaf_rn(0.08799999952316284f, F5_r00, F5_t0);
        const float _v63 = __fmaf_rn(0.08799999952316284f, F5_r10, F5_t1);
        const float _v64 = __fmaf_rn(0.08799999952316284f, F5_r20, F5_t2);
        float F6_s, F6_c; vg_sincos_ref(q[6], &F6_s, &F6_c);
        const float _v65 = __fmul_rn(F5_r00, F6_c);
        const float F6_r00 = __fmaf_rn(F5_r02, F6_s, _v65);
        const float _v67 = __fmul_rn((-F5_r00), F6_s);
        const float F6_r01 = __fmaf_rn(F5_r02, F6_c, _v67);
        const float F6_r02 = (-F5_r01);
        const float _v69 = __fmul_rn(F5_r10, F6_c);
        const float F6_r10 = __fmaf_rn(F5_r12, F6_s, _v69);
        const float _v71 = __fmul_rn((-F5_r10), F6_s);
        const float F6_r11 = __fmaf_rn(F5_r12, F6_c, _v71);
        const float F6_r12 = (-F5_r11);
        const float _v73 = __fmul_rn(F5_r20, F6_c);
        const float F6_r20 = __fmaf_rn(F5_r22, F6_s, _v73);
        const float _v75 = __fmul_rn((-F5_r20), F6_s);
        const float F6_r21 = __fmaf_rn(F5_r22, F6_c, _v75);
        const float F6_r22 = (-F5_r21);
        const float F6_t0 = _v62;
        const float F6_t1 = _v63;
        const float F6_t2 = _v64;
        float4 sa[18], sb[18];  // fine sphere scratch, reused by every check
        // environment: panda_rightfinger
        {
            const float _v77 = __fmaf_rn(F6_r00, -0.05409367009997368f, F6_t0);
            const float _v78 = __fmaf_rn(F6_r01, -0.05409367009997368f, _v77);
            const float c59_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v78);
            const float _v80 = __fmaf_rn(F6_r10, -0.05409367009997368f, F6_t1);
            const float _v81 = __fmaf_rn(F6_r11, -0.05409367009997368f, _v80);
            const float c59_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v81);
            const float _v83 = __fmaf_rn(F6_r20, -0.05409367009997368f, F6_t2);
            const float _v84 = __fmaf_rn(F6_r21, -0.05409367009997368f, _v83);
            const float c59_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v84);
            const unsigned need = ctx.env_hit(c59_x, c59_y, c59_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_0(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sa);
                if (vg::env_fine<2>(ctx, sa, need)) return;
            }
        }
        // environment: panda_leftfinger
        {
            const float _v86 = __fmaf_rn(F6_r00, 0.05409367009997368f, F6_t0);
            const float _v87 = __fmaf_rn(F6_r01, 0.05409367009997368f, _v86);
            const float c60_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v87);
            const float _v89 = __fmaf_rn(F6_r10, 0.05409367009997368f, F6_t1);
            const float _v90 = __fmaf_rn(F6_r11, 0.05409367009997368f, _v89);
            const float c60_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v90);
            const float _v92 = __fmaf_rn(F6_r20, 0.05409367009997368f, F6_t2);
            const float _v93 = __fmaf_rn(F6_r21, 0.05409367009997368f, _v92);
            const float c60_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v93);
            const unsigned need = ctx.env_hit(c60_x, c60_y, c60_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_1(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sa);
                if (vg::env_fine<2>(ctx, sa, need)) return;
            }
        }
        // environment: panda_hand
        {
            const float _v95 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
            const float _v96 = __fmaf_rn(F6_r01, 0.0f, _v95);
            const float c61_x = __fmaf_rn(F6_r02, 0.12920139729976654f, _v96);
            const float _v98 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
            const float _v99 = __fmaf_rn(F6_r11, 0.0f, _v98);
            const float c61_y = __fmaf_rn(F6_r12, 0.12920139729976654f, _v99);
            const float _v101 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
            const float _v102 = __fmaf_rn(F6_r21, 0.0f, _v101);
            const float c61_z = __fmaf_rn(F6_r22, 0.12920139729976654f, _v102);
            const unsigned need = ctx.env_hit(c61_x, c61_y, c61_z, 0.10398600995540619f, ctx.alive);
            if (need)
            {
                fine_2(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sa);
                if (vg::env_fine<18>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link7
        {
            const float _v104 = __fmaf_rn(F6_r00, 0.015300550498068333f, F6_t0);
            const float _v105 = __fmaf_rn(F6_r01, 0.015300550498068333f, _v104);
            const float c62_x = __fmaf_rn(F6_r02, 0.07459016144275665f, _v105);
            const float _v107 = __fmaf_rn(F6_r10, 0.015300550498068333f, F6_t1);
            const float _v108 = __fmaf_rn(F6_r11, 0.015300550498068333f, _v107);
            const float c62_y = __fmaf_rn(F6_r12, 0.07459016144275665f, _v108);
            const float _v110 = __fmaf_rn(F6_r20, 0.015300550498068333f, F6_t2);
            const float _v111 = __fmaf_rn(F6_r21, 0.015300550498068333f, _v110);
            const float c62_z = __fmaf_rn(F6_r22, 0.07459016144275665f, _v111);
            const unsigned need = ctx.env_hit(c62_x, c62_y, c62_z, 0.07211975008249283f, ctx.alive);
            if (need)
            {
                fine_3(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sa);
                if (vg::env_fine<5>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link6
        {
            const float _v113 = __fmaf_rn(F5_r00, 0.04243096336722374f, F5_t0);
            const float _v114 = __fmaf_rn(F5_r01, 0.014447699300944805f, _v113);
            const float c63_x = __fmaf_rn(F5_r02, 0.0f, _v114);
            const float _v116 = __fmaf_rn(F5_r10, 0.04243096336722374f, F5_t1);
            const float _v117 = __fmaf_rn(F5_r11, 0.014447699300944805f, _v116);
            const float c63_y = __fmaf_rn(F5_r12, 0.0f, _v117);
            const float _v119 = __fmaf_rn(F5_r20, 0.04243096336722374f, F5_t2);
            const float _v120 = __fmaf_rn(F5_r21, 0.014447699300944805f, _v119);
            const float c63_z = __fmaf_rn(F5_r22, 0.0f, _v120);
            const unsigned need = ctx.env_hit(c63_x, c63_y, c63_z, 0.09482324123382568f, ctx.alive);
            if (need)
            {
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<3>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link5
        {
            const float _v122 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v123 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v122);
            const float c64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v123);
            const float _v125 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v126 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v125);
            const float c64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v126);
            const float _v128 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v129 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v128);
            const float c64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v129);
            const unsigned need = ctx.env_hit(c64_x, c64_y, c64_z, 0.17621639370918274f, ctx.alive);
            if (need)
            {
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sa);
                if (vg::env_fine<12>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link4
        {
            const float _v131 = __fmaf_rn(F3_r00, -0.04144999757409096f, F3_t0);
            const float _v132 = __fmaf_rn(F3_r01, 0.04922187328338623f, _v131);
            const float c65_x = __fmaf_rn(F3_r02, 0.02891250140964985f, _v132);
            const float _v134 = __fmaf_rn(F3_r10, -0.04144999757409096f, F3_t1);
            const float _v135 = __fmaf_rn(F3_r11, 0.04922187328338623f, _v134);
            const float c65_y = __fmaf_rn(F3_r12, 0.02891250140964985f, _v135);
            const float _v137 = __fmaf_rn(F3_r20, -0.04144999757409096f, F3_t2);
            const float _v138 = __fmaf_rn(F3_r21, 0.04922187328338623f, _v137);
            const float c65_z = __fmaf_rn(F3_r22, 0.02891250140964985f, _v138);
            const unsigned need = ctx.env_hit(c65_x, c65_y, c65_z, 0.1264655739068985f, ctx.alive);
            if (need)
            {
                fine_6(F3_r00, F3_r01, F3_r02, F3_r10, F3_r11, F3_r12, F3_r20, F3_r21, F3_r22, F3_t0, F3_t1, F3_t2, sa);
                if (vg::env_fine<4>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link3
        {
            const float _v140 = __fmaf_rn(F2_r00, 0.038585785776376724f, F2_t0);
            const float _v141 = __fmaf_rn(F2_r01, 0.028939340263605118f, _v140);
            const float c66_x = __fmaf_rn(F2_r02, -0.05176776647567749f, _v141);
            const float _v143 = __fmaf_rn(F2_r10, 0.038585785776376724f, F2_t1);
            const float _v144 = __fmaf_rn(F2_r11, 0.028939340263605118f, _v143);
            const float c66_y = __fmaf_rn(F2_r12, -0.05176776647567749f, _v144);
            const float _v146 = __fmaf_rn(F2_r20, 0.038585785776376724f, F2_t2);
            const float _v147 = __fmaf_rn(F2_r21, 0.028939340263605118f, _v146);
            const float c66_z = __fmaf_rn(F2_r22, -0.05176776647567749f, _v147);
            const unsigned need = ctx.env_hit(c66_x, c66_y, c66_z, 0.12821067869663239f, ctx.alive);
            if (need)
            {
                fine_7(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r21, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                if (vg::env_fine<4>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link2
        {
            const float _v149 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
            const float _v150 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v149);
            const float c67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v150);
            const float _v152 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
            const float _v153 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v152);
            const float c67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v153);
            const float _v155 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
            const float _v156 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v155);
            const float c67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v156);
            const unsigned need = ctx.env_hit(c67_x, c67_y, c67_z, 0.15394146740436554f, ctx.alive);
            if (need)
            {
                fine_8(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r21, sa);
                if (vg::env_fine<4>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link1
        {
            const float _v158 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v159 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v158);
            const float c68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v159);
            const float _v161 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v162 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v161);
            const float c68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v162);
            const float _v164 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v165 = __fmaf_rn(0.0f, -0.03999999910593033f, _v164);
            const float c68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v165);
            const unsigned need = ctx.env_hit(c68_x, c68_y, c68_z, 0.15394146740436554f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                if (vg::env_fine<4>(ctx, sa, need)) return;
            }
        }
        // environment: panda_link0
        {
            const float _v167 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v168 = __fmaf_rn(0.0f, 0.0f, _v167);
            const float c69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v168);
            const float _v170 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v171 = __fmaf_rn(1.0f, 0.0f, _v170);
            const float c69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v171);
            const float _v173 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v174 = __fmaf_rn(0.0f, 0.0f, _v173);
            const float c69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v174);
            const unsigned need = ctx.env_hit(c69_x, c69_y, c69_z, 0.07999999821186066f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // self: panda_link0 vs. panda_link5
        {
            const float _v176 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v177 = __fmaf_rn(0.0f, 0.0f, _v176);
            const float ca69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v177);
            const float _v179 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v180 = __fmaf_rn(1.0f, 0.0f, _v179);
            const float ca69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v180);
            const float _v182 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v183 = __fmaf_rn(0.0f, 0.0f, _v182);
            const float ca69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v183);
            const float _v185 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v186 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v185);
            const float cb64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v186);
            const float _v188 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v189 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v188);
            const float cb64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v189);
            const float _v191 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v192 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v191);
            const float cb64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v192);
            const unsigned need = ctx.self_hit(ca69_x, ca69_y, ca69_z, 0.07999999821186066f, cb64_x, cb64_y, cb64_z, 0.17621639370918274f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<1, 12>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link0 vs. panda_link6
        {
            const float _v194 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v195 = __fmaf_rn(0.0f, 0.0f, _v194);
            const float ca69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v195);
            const float _v197 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v198 = __fmaf_rn(1.0f, 0.0f, _v197);
            const float ca69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v198);
            const float _v200 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v201 = __fmaf_rn(0.0f, 0.0f, _v200);
            const float ca69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v201);
            const float _v203 = __fmaf_rn(F5_r00, 0.04243096336722374f, F5_t0);
            const float _v204 = __fmaf_rn(F5_r01, 0.014447699300944805f, _v203);
            const float cb63_x = __fmaf_rn(F5_r02, 0.0f, _v204);
            const float _v206 = __fmaf_rn(F5_r10, 0.04243096336722374f, F5_t1);
            const float _v207 = __fmaf_rn(F5_r11, 0.014447699300944805f, _v206);
            const float cb63_y = __fmaf_rn(F5_r12, 0.0f, _v207);
            const float _v209 = __fmaf_rn(F5_r20, 0.04243096336722374f, F5_t2);
            const float _v210 = __fmaf_rn(F5_r21, 0.014447699300944805f, _v209);
            const float cb63_z = __fmaf_rn(F5_r22, 0.0f, _v210);
            const unsigned need = ctx.self_hit(ca69_x, ca69_y, ca69_z, 0.07999999821186066f, cb63_x, cb63_y, cb63_z, 0.09482324123382568f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link0 vs. panda_link7
        {
            const float _v212 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v213 = __fmaf_rn(0.0f, 0.0f, _v212);
            const float ca69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v213);
            const float _v215 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v216 = __fmaf_rn(1.0f, 0.0f, _v215);
            const float ca69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v216);
            const float _v218 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v219 = __fmaf_rn(0.0f, 0.0f, _v218);
            const float ca69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v219);
            const float _v221 = __fmaf_rn(F6_r00, 0.015300550498068333f, F6_t0);
            const float _v222 = __fmaf_rn(F6_r01, 0.015300550498068333f, _v221);
            const float cb62_x = __fmaf_rn(F6_r02, 0.07459016144275665f, _v222);
            const float _v224 = __fmaf_rn(F6_r10, 0.015300550498068333f, F6_t1);
            const float _v225 = __fmaf_rn(F6_r11, 0.015300550498068333f, _v224);
            const float cb62_y = __fmaf_rn(F6_r12, 0.07459016144275665f, _v225);
            const float _v227 = __fmaf_rn(F6_r20, 0.015300550498068333f, F6_t2);
            const float _v228 = __fmaf_rn(F6_r21, 0.015300550498068333f, _v227);
            const float cb62_z = __fmaf_rn(F6_r22, 0.07459016144275665f, _v228);
            const unsigned need = ctx.self_hit(ca69_x, ca69_y, ca69_z, 0.07999999821186066f, cb62_x, cb62_y, cb62_z, 0.07211975008249283f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                fine_3(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<1, 5>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link0 vs. panda_hand
        {
            const float _v230 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v231 = __fmaf_rn(0.0f, 0.0f, _v230);
            const float ca69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v231);
            const float _v233 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v234 = __fmaf_rn(1.0f, 0.0f, _v233);
            const float ca69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v234);
            const float _v236 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v237 = __fmaf_rn(0.0f, 0.0f, _v236);
            const float ca69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v237);
            const float _v239 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
            const float _v240 = __fmaf_rn(F6_r01, 0.0f, _v239);
            const float cb61_x = __fmaf_rn(F6_r02, 0.12920139729976654f, _v240);
            const float _v242 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
            const float _v243 = __fmaf_rn(F6_r11, 0.0f, _v242);
            const float cb61_y = __fmaf_rn(F6_r12, 0.12920139729976654f, _v243);
            const float _v245 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
            const float _v246 = __fmaf_rn(F6_r21, 0.0f, _v245);
            const float cb61_z = __fmaf_rn(F6_r22, 0.12920139729976654f, _v246);
            const unsigned need = ctx.self_hit(ca69_x, ca69_y, ca69_z, 0.07999999821186066f, cb61_x, cb61_y, cb61_z, 0.10398600995540619f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                fine_2(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<1, 18>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link0 vs. panda_leftfinger
        {
            const float _v248 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v249 = __fmaf_rn(0.0f, 0.0f, _v248);
            const float ca69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v249);
            const float _v251 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v252 = __fmaf_rn(1.0f, 0.0f, _v251);
            const float ca69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v252);
            const float _v254 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v255 = __fmaf_rn(0.0f, 0.0f, _v254);
            const float ca69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v255);
            const float _v257 = __fmaf_rn(F6_r00, 0.05409367009997368f, F6_t0);
            const float _v258 = __fmaf_rn(F6_r01, 0.05409367009997368f, _v257);
            const float cb60_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v258);
            const float _v260 = __fmaf_rn(F6_r10, 0.05409367009997368f, F6_t1);
            const float _v261 = __fmaf_rn(F6_r11, 0.05409367009997368f, _v260);
            const float cb60_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v261);
            const float _v263 = __fmaf_rn(F6_r20, 0.05409367009997368f, F6_t2);
            const float _v264 = __fmaf_rn(F6_r21, 0.05409367009997368f, _v263);
            const float cb60_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v264);
            const unsigned need = ctx.self_hit(ca69_x, ca69_y, ca69_z, 0.07999999821186066f, cb60_x, cb60_y, cb60_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                fine_1(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link0 vs. panda_rightfinger
        {
            const float _v266 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v267 = __fmaf_rn(0.0f, 0.0f, _v266);
            const float ca69_x = __fmaf_rn(0.0f, 0.05000000074505806f, _v267);
            const float _v269 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v270 = __fmaf_rn(1.0f, 0.0f, _v269);
            const float ca69_y = __fmaf_rn(0.0f, 0.05000000074505806f, _v270);
            const float _v272 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v273 = __fmaf_rn(0.0f, 0.0f, _v272);
            const float ca69_z = __fmaf_rn(1.0f, 0.05000000074505806f, _v273);
            const float _v275 = __fmaf_rn(F6_r00, -0.05409367009997368f, F6_t0);
            const float _v276 = __fmaf_rn(F6_r01, -0.05409367009997368f, _v275);
            const float cb59_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v276);
            const float _v278 = __fmaf_rn(F6_r10, -0.05409367009997368f, F6_t1);
            const float _v279 = __fmaf_rn(F6_r11, -0.05409367009997368f, _v278);
            const float cb59_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v279);
            const float _v281 = __fmaf_rn(F6_r20, -0.05409367009997368f, F6_t2);
            const float _v282 = __fmaf_rn(F6_r21, -0.05409367009997368f, _v281);
            const float cb59_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v282);
            const unsigned need = ctx.self_hit(ca69_x, ca69_y, ca69_z, 0.07999999821186066f, cb59_x, cb59_y, cb59_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_10(sa);
                fine_0(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link1 vs. panda_link5
        {
            const float _v284 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v285 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v284);
            const float ca68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v285);
            const float _v287 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v288 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v287);
            const float ca68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v288);
            const float _v290 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v291 = __fmaf_rn(0.0f, -0.03999999910593033f, _v290);
            const float ca68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v291);
            const float _v293 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v294 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v293);
            const float cb64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v294);
            const float _v296 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v297 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v296);
            const float cb64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v297);
            const float _v299 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v300 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v299);
            const float cb64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v300);
            const unsigned need = ctx.self_hit(ca68_x, ca68_y, ca68_z, 0.15394146740436554f, cb64_x, cb64_y, cb64_z, 0.17621639370918274f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<4, 12>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link1 vs. panda_link6
        {
            const float _v302 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v303 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v302);
            const float ca68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v303);
            const float _v305 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v306 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v305);
            const float ca68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v306);
            const float _v308 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v309 = __fmaf_rn(0.0f, -0.03999999910593033f, _v308);
            const float ca68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v309);
            const float _v311 = __fmaf_rn(F5_r00, 0.04243096336722374f, F5_t0);
            const float _v312 = __fmaf_rn(F5_r01, 0.014447699300944805f, _v311);
            const float cb63_x = __fmaf_rn(F5_r02, 0.0f, _v312);
            const float _v314 = __fmaf_rn(F5_r10, 0.04243096336722374f, F5_t1);
            const float _v315 = __fmaf_rn(F5_r11, 0.014447699300944805f, _v314);
            const float cb63_y = __fmaf_rn(F5_r12, 0.0f, _v315);
            const float _v317 = __fmaf_rn(F5_r20, 0.04243096336722374f, F5_t2);
            const float _v318 = __fmaf_rn(F5_r21, 0.014447699300944805f, _v317);
            const float cb63_z = __fmaf_rn(F5_r22, 0.0f, _v318);
            const unsigned need = ctx.self_hit(ca68_x, ca68_y, ca68_z, 0.15394146740436554f, cb63_x, cb63_y, cb63_z, 0.09482324123382568f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<4, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link1 vs. panda_link7
        {
            const float _v320 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v321 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v320);
            const float ca68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v321);
            const float _v323 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v324 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v323);
            const float ca68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v324);
            const float _v326 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v327 = __fmaf_rn(0.0f, -0.03999999910593033f, _v326);
            const float ca68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v327);
            const float _v329 = __fmaf_rn(F6_r00, 0.015300550498068333f, F6_t0);
            const float _v330 = __fmaf_rn(F6_r01, 0.015300550498068333f, _v329);
            const float cb62_x = __fmaf_rn(F6_r02, 0.07459016144275665f, _v330);
            const float _v332 = __fmaf_rn(F6_r10, 0.015300550498068333f, F6_t1);
            const float _v333 = __fmaf_rn(F6_r11, 0.015300550498068333f, _v332);
            const float cb62_y = __fmaf_rn(F6_r12, 0.07459016144275665f, _v333);
            const float _v335 = __fmaf_rn(F6_r20, 0.015300550498068333f, F6_t2);
            const float _v336 = __fmaf_rn(F6_r21, 0.015300550498068333f, _v335);
            const float cb62_z = __fmaf_rn(F6_r22, 0.07459016144275665f, _v336);
            const unsigned need = ctx.self_hit(ca68_x, ca68_y, ca68_z, 0.15394146740436554f, cb62_x, cb62_y, cb62_z, 0.07211975008249283f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_3(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 5>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link1 vs. panda_hand
        {
            const float _v338 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v339 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v338);
            const float ca68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v339);
            const float _v341 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v342 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v341);
            const float ca68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v342);
            const float _v344 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v345 = __fmaf_rn(0.0f, -0.03999999910593033f, _v344);
            const float ca68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v345);
            const float _v347 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
            const float _v348 = __fmaf_rn(F6_r01, 0.0f, _v347);
            const float cb61_x = __fmaf_rn(F6_r02, 0.12920139729976654f, _v348);
            const float _v350 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
            const float _v351 = __fmaf_rn(F6_r11, 0.0f, _v350);
            const float cb61_y = __fmaf_rn(F6_r12, 0.12920139729976654f, _v351);
            const float _v353 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
            const float _v354 = __fmaf_rn(F6_r21, 0.0f, _v353);
            const float cb61_z = __fmaf_rn(F6_r22, 0.12920139729976654f, _v354);
            const unsigned need = ctx.self_hit(ca68_x, ca68_y, ca68_z, 0.15394146740436554f, cb61_x, cb61_y, cb61_z, 0.10398600995540619f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_2(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 18>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link1 vs. panda_leftfinger
        {
            const float _v356 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v357 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v356);
            const float ca68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v357);
            const float _v359 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v360 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v359);
            const float ca68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v360);
            const float _v362 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v363 = __fmaf_rn(0.0f, -0.03999999910593033f, _v362);
            const float ca68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v363);
            const float _v365 = __fmaf_rn(F6_r00, 0.05409367009997368f, F6_t0);
            const float _v366 = __fmaf_rn(F6_r01, 0.05409367009997368f, _v365);
            const float cb60_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v366);
            const float _v368 = __fmaf_rn(F6_r10, 0.05409367009997368f, F6_t1);
            const float _v369 = __fmaf_rn(F6_r11, 0.05409367009997368f, _v368);
            const float cb60_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v369);
            const float _v371 = __fmaf_rn(F6_r20, 0.05409367009997368f, F6_t2);
            const float _v372 = __fmaf_rn(F6_r21, 0.05409367009997368f, _v371);
            const float cb60_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v372);
            const unsigned need = ctx.self_hit(ca68_x, ca68_y, ca68_z, 0.15394146740436554f, cb60_x, cb60_y, cb60_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_1(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link1 vs. panda_rightfinger
        {
            const float _v374 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v375 = __fmaf_rn(F0_r01, -0.03999999910593033f, _v374);
            const float ca68_x = __fmaf_rn(0.0f, -0.08500000089406967f, _v375);
            const float _v377 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v378 = __fmaf_rn(F0_r11, -0.03999999910593033f, _v377);
            const float ca68_y = __fmaf_rn(0.0f, -0.08500000089406967f, _v378);
            const float _v380 = __fmaf_rn(0.0f, 0.0f, 0.3330000042915344f);
            const float _v381 = __fmaf_rn(0.0f, -0.03999999910593033f, _v380);
            const float ca68_z = __fmaf_rn(1.0f, -0.08500000089406967f, _v381);
            const float _v383 = __fmaf_rn(F6_r00, -0.05409367009997368f, F6_t0);
            const float _v384 = __fmaf_rn(F6_r01, -0.05409367009997368f, _v383);
            const float cb59_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v384);
            const float _v386 = __fmaf_rn(F6_r10, -0.05409367009997368f, F6_t1);
            const float _v387 = __fmaf_rn(F6_r11, -0.05409367009997368f, _v386);
            const float cb59_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v387);
            const float _v389 = __fmaf_rn(F6_r20, -0.05409367009997368f, F6_t2);
            const float _v390 = __fmaf_rn(F6_r21, -0.05409367009997368f, _v389);
            const float cb59_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v390);
            const unsigned need = ctx.self_hit(ca68_x, ca68_y, ca68_z, 0.15394146740436554f, cb59_x, cb59_y, cb59_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_9(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_0(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link2 vs. panda_link5
        {
            const float _v392 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
            const float _v393 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v392);
            const float ca67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v393);
            const float _v395 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
            const float _v396 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v395);
            const float ca67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v396);
            const float _v398 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
            const float _v399 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v398);
            const float ca67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v399);
            const float _v401 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v402 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v401);
            const float cb64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v402);
            const float _v404 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v405 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v404);
            const float cb64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v405);
            const float _v407 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v408 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v407);
            const float cb64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v408);
            const unsigned need = ctx.self_hit(ca67_x, ca67_y, ca67_z, 0.15394146740436554f, cb64_x, cb64_y, cb64_z, 0.17621639370918274f, ctx.alive);
            if (need)
            {
                fine_8(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r21, sa);
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<4, 12>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link2 vs. panda_link7
        {
            const float _v410 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
            const float _v411 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v410);
            const float ca67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v411);
            const float _v413 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
            const float _v414 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v413);
            const float ca67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v414);
            const float _v416 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
            const float _v417 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v416);
            const float ca67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v417);
            const float _v419 = __fmaf_rn(F6_r00, 0.015300550498068333f, F6_t0);
            const float _v420 = __fmaf_rn(F6_r01, 0.015300550498068333f, _v419);
            const float cb62_x = __fmaf_rn(F6_r02, 0.07459016144275665f, _v420);
            const float _v422 = __fmaf_rn(F6_r10, 0.015300550498068333f, F6_t1);
            const float _v423 = __fmaf_rn(F6_r11, 0.015300550498068333f, _v422);
            const float cb62_y = __fmaf_rn(F6_r12, 0.07459016144275665f, _v423);
            const float _v425 = __fmaf_rn(F6_r20, 0.015300550498068333f, F6_t2);
            const float _v426 = __fmaf_rn(F6_r21, 0.015300550498068333f, _v425);
            const float cb62_z = __fmaf_rn(F6_r22, 0.07459016144275665f, _v426);
            const unsigned need = ctx.self_hit(ca67_x, ca67_y, ca67_z, 0.15394146740436554f, cb62_x, cb62_y, cb62_z, 0.07211975008249283f, ctx.alive);
            if (need)
            {
                fine_8(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r21, sa);
                fine_3(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 5>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link2 vs. panda_hand
        {
            const float _v428 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
            const float _v429 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v428);
            const float ca67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v429);
            const float _v431 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
            const float _v432 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v431);
            const float ca67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v432);
            const float _v434 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
            const float _v435 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v434);
            const float ca67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v435);
            const float _v437 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
            const float _v438 = __fmaf_rn(F6_r01, 0.0f, _v437);
            const float cb61_x = __fmaf_rn(F6_r02, 0.12920139729976654f, _v438);
            const float _v440 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
            const float _v441 = __fmaf_rn(F6_r11, 0.0f, _v440);
            const float cb61_y = __fmaf_rn(F6_r12, 0.12920139729976654f, _v441);
            const float _v443 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
            const float _v444 = __fmaf_rn(F6_r21, 0.0f, _v443);
            const float cb61_z = __fmaf_rn(F6_r22, 0.12920139729976654f, _v444);
            const unsigned need = ctx.self_hit(ca67_x, ca67_y, ca67_z, 0.15394146740436554f, cb61_x, cb61_y, cb61_z, 0.10398600995540619f, ctx.alive);
            if (need)
            {
                fine_8(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r21, sa);
                fine_2(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 18>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link2 vs. panda_leftfinger
        {
            const float _v446 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
            const float _v447 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v446);
            const float ca67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v447);
            const float _v449 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
            const float _v450 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v449);
            const float ca67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v450);
            const float _v452 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
            const float _v453 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v452);
            const float ca67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v453);
            const float _v455 = __fmaf_rn(F6_r00, 0.05409367009997368f, F6_t0);
            const float _v456 = __fmaf_rn(F6_r01, 0.05409367009997368f, _v455);
            const float cb60_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v456);
            const float _v458 = __fmaf_rn(F6_r10, 0.05409367009997368f, F6_t1);
            const float _v459 = __fmaf_rn(F6_r11, 0.05409367009997368f, _v458);
            const float cb60_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v459);
            const float _v461 = __fmaf_rn(F6_r20, 0.05409367009997368f, F6_t2);
            const float _v462 = __fmaf_rn(F6_r21, 0.05409367009997368f, _v461);
            const float cb60_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v462);
            const unsigned need = ctx.self_hit(ca67_x, ca67_y, ca67_z, 0.15394146740436554f, cb60_x, cb60_y, cb60_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_8(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r21, sa);
                fine_1(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link2 vs. panda_rightfinger
        {
            const float _v464 = __fmaf_rn(F1_r00, 0.0f, 0.0f);
            const float _v465 = __fmaf_rn(F1_r01, -0.08500000089406967f, _v464);
            const float ca67_x = __fmaf_rn(F1_r02, 0.03999999910593033f, _v465);
            const float _v467 = __fmaf_rn(F1_r10, 0.0f, 0.0f);
            const float _v468 = __fmaf_rn(F1_r11, -0.08500000089406967f, _v467);
            const float ca67_y = __fmaf_rn(F1_r12, 0.03999999910593033f, _v468);
            const float _v470 = __fmaf_rn(F1_r20, 0.0f, 0.3330000042915344f);
            const float _v471 = __fmaf_rn(F1_r21, -0.08500000089406967f, _v470);
            const float ca67_z = __fmaf_rn(0.0f, 0.03999999910593033f, _v471);
            const float _v473 = __fmaf_rn(F6_r00, -0.05409367009997368f, F6_t0);
            const float _v474 = __fmaf_rn(F6_r01, -0.05409367009997368f, _v473);
            const float cb59_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v474);
            const float _v476 = __fmaf_rn(F6_r10, -0.05409367009997368f, F6_t1);
            const float _v477 = __fmaf_rn(F6_r11, -0.05409367009997368f, _v476);
            const float cb59_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v477);
            const float _v479 = __fmaf_rn(F6_r20, -0.05409367009997368f, F6_t2);
            const float _v480 = __fmaf_rn(F6_r21, -0.05409367009997368f, _v479);
            const float cb59_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v480);
            const unsigned need = ctx.self_hit(ca67_x, ca67_y, ca67_z, 0.15394146740436554f, cb59_x, cb59_y, cb59_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_8(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r21, sa);
                fine_0(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<4, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link5 vs. panda_link7
        {
            const float _v482 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v483 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v482);
            const float ca64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v483);
            const float _v485 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v486 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v485);
            const float ca64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v486);
            const float _v488 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v489 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v488);
            const float ca64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v489);
            const float _v491 = __fmaf_rn(F6_r00, 0.015300550498068333f, F6_t0);
            const float _v492 = __fmaf_rn(F6_r01, 0.015300550498068333f, _v491);
            const float cb62_x = __fmaf_rn(F6_r02, 0.07459016144275665f, _v492);
            const float _v494 = __fmaf_rn(F6_r10, 0.015300550498068333f, F6_t1);
            const float _v495 = __fmaf_rn(F6_r11, 0.015300550498068333f, _v494);
            const float cb62_y = __fmaf_rn(F6_r12, 0.07459016144275665f, _v495);
            const float _v497 = __fmaf_rn(F6_r20, 0.015300550498068333f, F6_t2);
            const float _v498 = __fmaf_rn(F6_r21, 0.015300550498068333f, _v497);
            const float cb62_z = __fmaf_rn(F6_r22, 0.07459016144275665f, _v498);
            const unsigned need = ctx.self_hit(ca64_x, ca64_y, ca64_z, 0.17621639370918274f, cb62_x, cb62_y, cb62_z, 0.07211975008249283f, ctx.alive);
            if (need)
            {
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sa);
                fine_3(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<12, 5>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link5 vs. panda_hand
        {
            const float _v500 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v501 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v500);
            const float ca64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v501);
            const float _v503 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v504 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v503);
            const float ca64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v504);
            const float _v506 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v507 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v506);
            const float ca64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v507);
            const float _v509 = __fmaf_rn(F6_r00, 0.0f, F6_t0);
            const float _v510 = __fmaf_rn(F6_r01, 0.0f, _v509);
            const float cb61_x = __fmaf_rn(F6_r02, 0.12920139729976654f, _v510);
            const float _v512 = __fmaf_rn(F6_r10, 0.0f, F6_t1);
            const float _v513 = __fmaf_rn(F6_r11, 0.0f, _v512);
            const float cb61_y = __fmaf_rn(F6_r12, 0.12920139729976654f, _v513);
            const float _v515 = __fmaf_rn(F6_r20, 0.0f, F6_t2);
            const float _v516 = __fmaf_rn(F6_r21, 0.0f, _v515);
            const float cb61_z = __fmaf_rn(F6_r22, 0.12920139729976654f, _v516);
            const unsigned need = ctx.self_hit(ca64_x, ca64_y, ca64_z, 0.17621639370918274f, cb61_x, cb61_y, cb61_z, 0.10398600995540619f, ctx.alive);
            if (need)
            {
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sa);
                fine_2(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<12, 18>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link5 vs. panda_leftfinger
        {
            const float _v518 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v519 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v518);
            const float ca64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v519);
            const float _v521 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v522 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v521);
            const float ca64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v522);
            const float _v524 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v525 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v524);
            const float ca64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v525);
            const float _v527 = __fmaf_rn(F6_r00, 0.05409367009997368f, F6_t0);
            const float _v528 = __fmaf_rn(F6_r01, 0.05409367009997368f, _v527);
            const float cb60_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v528);
            const float _v530 = __fmaf_rn(F6_r10, 0.05409367009997368f, F6_t1);
            const float _v531 = __fmaf_rn(F6_r11, 0.05409367009997368f, _v530);
            const float cb60_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v531);
            const float _v533 = __fmaf_rn(F6_r20, 0.05409367009997368f, F6_t2);
            const float _v534 = __fmaf_rn(F6_r21, 0.05409367009997368f, _v533);
            const float cb60_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v534);
            const unsigned need = ctx.self_hit(ca64_x, ca64_y, ca64_z, 0.17621639370918274f, cb60_x, cb60_y, cb60_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sa);
                fine_1(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<12, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: panda_link5 vs. panda_rightfinger
        {
            const float _v536 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v537 = __fmaf_rn(F4_r01, 0.03750000149011612f, _v536);
            const float ca64_x = __fmaf_rn(F4_r02, -0.10999999940395355f, _v537);
            const float _v539 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v540 = __fmaf_rn(F4_r11, 0.03750000149011612f, _v539);
            const float ca64_y = __fmaf_rn(F4_r12, -0.10999999940395355f, _v540);
            const float _v542 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v543 = __fmaf_rn(F4_r21, 0.03750000149011612f, _v542);
            const float ca64_z = __fmaf_rn(F4_r22, -0.10999999940395355f, _v543);
            const float _v545 = __fmaf_rn(F6_r00, -0.05409367009997368f, F6_t0);
            const float _v546 = __fmaf_rn(F6_r01, -0.05409367009997368f, _v545);
            const float cb59_x = __fmaf_rn(F6_r02, 0.19840000569820404f, _v546);
            const float _v548 = __fmaf_rn(F6_r10, -0.05409367009997368f, F6_t1);
            const float _v549 = __fmaf_rn(F6_r11, -0.05409367009997368f, _v548);
            const float cb59_y = __fmaf_rn(F6_r12, 0.19840000569820404f, _v549);
            const float _v551 = __fmaf_rn(F6_r20, -0.05409367009997368f, F6_t2);
            const float _v552 = __fmaf_rn(F6_r21, -0.05409367009997368f, _v551);
            const float cb59_z = __fmaf_rn(F6_r22, 0.19840000569820404f, _v552);
            const unsigned need = ctx.self_hit(ca64_x, ca64_y, ca64_z, 0.17621639370918274f, cb59_x, cb59_y, cb59_z, 0.023543396964669228f, ctx.alive);
            if (need)
            {
                fine_5(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sa);
                fine_0(F6_r00, F6_r01, F6_r02, F6_r10, F6_r11, F6_r12, F6_r20, F6_r21, F6_r22, F6_t0, F6_t1, F6_t2, sb);
                if (vg::self_cross<12, 2>(ctx, sa, sb, need)) return;
            }
        }
    }
};
}  // namespace vg::robots
