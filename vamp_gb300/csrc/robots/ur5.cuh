// Generated by vamp_gb300/robotgen/codegen.py from vamp_gb300/robots/ur5.json. Do not edit.
//
// FP32 forward kinematics and the fkcc check schedule of the ur5 robot, one configuration
// per thread.  Schedule order follows the reference's generated Robot::fkcc
// (src/impl/vamp/robots/ur5.hh): environment checks link by link, each a coarse link sphere
// gating that link's fine spheres, then self-collision link pairs, a coarse pair gating the
// cross product of the two links' fine spheres.  Schedule form: straight-line.
#pragma once

#include "../vg_check.cuh"

namespace vg::robots
{
struct Ur5
{
    static constexpr const char *kName = "ur5";
    static constexpr int kDim = 6;
    static constexpr int kFine = 40;
    static constexpr int kSlots = 57;
    static constexpr int kFrames = 7;
    static constexpr int kResolution = 32;
    static constexpr float kMinRadius = 0.014999999664723873f;
    static constexpr float kMaxRadius = 0.07999999821186066f;
    static constexpr float kScaleM[6] = {6.2831854820251465f, 6.2831854820251465f, 6.2831854820251465f, 6.2831854820251465f, 6.2831854820251465f, 6.2831854820251465f};
    static constexpr float kScaleA[6] = {-3.1415927410125732f, -3.1415927410125732f, -3.1415927410125732f, -3.1415927410125732f, -3.1415927410125732f, -3.1415927410125732f};

    // Every sphere slot: fine spheres 0..kFine-1, then the coarse sphere of each checked link.
    static __device__ __forceinline__ void spheres(const float *q, float *out)
    {
        float F0_s, F0_c; vg_sincos_ref(q[0], &F0_s, &F0_c);
        const float _v0 = __fmul_rn(0.0007963267271406949f, F0_c);
        const float F0_r00 = __fmaf_rn(-0.9999997019767761f, F0_s, _v0);
        const float _v2 = __fmul_rn(-0.0007963267271406949f, F0_s);
        const float F0_r01 = __fmaf_rn(-0.9999997019767761f, F0_c, _v2);
        const float _v4 = __fmul_rn(0.9999997019767761f, F0_c);
        const float F0_r10 = __fmaf_rn(0.0007963267271406949f, F0_s, _v4);
        const float _v6 = __fmul_rn(-0.9999997019767761f, F0_s);
        const float F0_r11 = __fmaf_rn(0.0007963267271406949f, F0_c, _v6);
        const float _v8 = __fmul_rn(0.1358499974012375f, F0_r01);
        const float _v9 = __fmul_rn(0.1358499974012375f, F0_r11);
        const float _v10 = __fmul_rn(1.7948965647107684e-09f, F0_r00);
        const float _v11 = __fmul_rn(1.7948965647107684e-09f, F0_r10);
        float F1_s, F1_c; vg_sincos_ref(q[1], &F1_s, &F1_c);
        const float _v12 = __fmul_rn(_v10, F1_c);
        const float F1_r00 = __fmaf_rn((-F0_r00), F1_s, _v12);
        const float F1_r01 = F0_r01;
        const float _v14 = __fmul_rn(_v10, F1_s);
        const float F1_r02 = __fmaf_rn(F0_r00, F1_c, _v14);
        const float _v16 = __fmul_rn(_v11, F1_c);
        const float F1_r10 = __fmaf_rn((-F0_r10), F1_s, _v16);
        const float F1_r11 = F0_r11;
        const float _v18 = __fmul_rn(_v11, F1_s);
        const float F1_r12 = __fmaf_rn(F0_r10, F1_c, _v18);
        const float F1_r20 = __fmaf_rn(-1.7948965647107684e-09f, F1_s, (-F1_c));
        const float F1_r22 = __fmaf_rn(1.7948965647107684e-09f, F1_c, (-F1_s));
        const float F1_t0 = _v8;
        const float F1_t1 = _v9;
        const float _v22 = __fmaf_rn(-0.11969999969005585f, F1_r01, F1_t0);
        const float _v23 = __fmaf_rn(0.42500001192092896f, F1_r02, _v22);
        const float _v24 = __fmaf_rn(-0.11969999969005585f, F1_r11, F1_t1);
        const float _v25 = __fmaf_rn(0.42500001192092896f, F1_r12, _v24);
        const float _v26 = __fmaf_rn(0.42500001192092896f, F1_r22, 1.0035589933395386f);
        float F2_s, F2_c; vg_sincos_ref(q[2], &F2_s, &F2_c);
        const float _v27 = __fmul_rn(F1_r00, F2_c);
        const float F2_r00 = __fmaf_rn((-F1_r02), F2_s, _v27);
        const float F2_r01 = F1_r01;
        const float _v29 = __fmul_rn(F1_r00, F2_s);
        const float F2_r02 = __fmaf_rn(F1_r02, F2_c, _v29);
        const float _v31 = __fmul_rn(F1_r10, F2_c);
        const float F2_r10 = __fmaf_rn((-F1_r12), F2_s, _v31);
        const float F2_r11 = F1_r11;
        const float _v33 = __fmul_rn(F1_r10, F2_s);
        const float F2_r12 = __fmaf_rn(F1_r12, F2_c, _v33);
        const float _v35 = __fmul_rn(F1_r20, F2_c);
        const float F2_r20 = __fmaf_rn((-F1_r22), F2_s, _v35);
        const float _v37 = __fmul_rn(F1_r20, F2_s);
        const float F2_r22 = __fmaf_rn(F1_r22, F2_c, _v37);
        const float F2_t0 = _v23;
        const float F2_t1 = _v25;
        const float F2_t2 = _v26;
        const float _v39 = __fmaf_rn(0.3922500014305115f, F2_r02, F2_t0);
        const float _v40 = __fmaf_rn(0.3922500014305115f, F2_r12, F2_t1);
        const float _v41 = __fmaf_rn(0.3922500014305115f, F2_r22, F2_t2);
        const float _v42 = __fmaf_rn(1.7948965647107684e-09f, F2_r00, (-F2_r02));
        const float _v43 = __fmaf_rn(1.7948965647107684e-09f, F2_r02, F2_r00);
        const float _v44 = __fmaf_rn(1.7948965647107684e-09f, F2_r10, (-F2_r12));
        const float _v45 = __fmaf_rn(1.7948965647107684e-09f, F2_r12, F2_r10);
        const float _v46 = __fmaf_rn(1.7948965647107684e-09f, F2_r20, (-F2_r22));
        const float _v47 = __fmaf_rn(1.7948965647107684e-09f, F2_r22, F2_r20);
        float F3_s, F3_c; vg_sincos_ref(q[3], &F3_s, &F3_c);
        const float _v48 = __fmul_rn(_v42, F3_c);
        const float F3_r00 = __fmaf_rn((-_v43), F3_s, _v48);
        const float F3_r01 = F2_r01;
        const float _v50 = __fmul_rn(_v42, F3_s);
        const float F3_r02 = __fmaf_rn(_v43, F3_c, _v50);
        const float _v52 = __fmul_rn(_v44, F3_c);
        const float F3_r10 = __fmaf_rn((-_v45), F3_s, _v52);
        const float F3_r11 = F2_r11;
        const float _v54 = __fmul_rn(_v44, F3_s);
        const float F3_r12 = __fmaf_rn(_v45, F3_c, _v54);
        const float _v56 = __fmul_rn(_v46, F3_c);
        const float F3_r20 = __fmaf_rn((-_v47), F3_s, _v56);
        const float _v58 = __fmul_rn(_v46, F3_s);
        const float F3_r22 = __fmaf_rn(_v47, F3_c, _v58);
        const float F3_t0 = _v39;
        const float F3_t1 = _v40;
        const float F3_t2 = _v41;
        const float _v60 = __fmaf_rn(0.09300000220537186f, F3_r01, F3_t0);
        const float _v61 = __fmaf_rn(0.09300000220537186f, F3_r11, F3_t1);
        float F4_s, F4_c; vg_sincos_ref(q[4], &F4_s, &F4_c);
        const float _v62 = __fmul_rn(F3_r00, F4_c);
        const float F4_r00 = __fmaf_rn(F3_r01, F4_s, _v62);
        const float _v64 = __fmul_rn((-F3_r00), F4_s);
        const float F4_r01 = __fmaf_rn(F3_r01, F4_c, _v64);
        const float F4_r02 = F3_r02;
        const float _v66 = __fmul_rn(F3_r10, F4_c);
        const float F4_r10 = __fmaf_rn(F3_r11, F4_s, _v66);
        const float _v68 = __fmul_rn((-F3_r10), F4_s);
        const float F4_r11 = __fmaf_rn(F3_r11, F4_c, _v68);
        const float F4_r12 = F3_r12;
        const float F4_r20 = __fmul_rn(F3_r20, F4_c);
        const float F4_r21 = __fmul_rn((-F3_r20), F4_s);
        const float F4_r22 = F3_r22;
        const float F4_t0 = _v60;
        const float F4_t1 = _v61;
        const float F4_t2 = F3_t2;
        const float _v72 = __fmaf_rn(0.09465000033378601f, F4_r02, F4_t0);
        const float _v73 = __fmaf_rn(0.09465000033378601f, F4_r12, F4_t1);
        const float _v74 = __fmaf_rn(0.09465000033378601f, F4_r22, F4_t2);
        float F5_s, F5_c; vg_sincos_ref(q[5], &F5_s, &F5_c);
        const float _v75 = __fmul_rn(F4_r00, F5_c);
        const float F5_r00 = __fmaf_rn((-F4_r02), F5_s, _v75);
        const float F5_r01 = F4_r01;
        const float _v77 = __fmul_rn(F4_r00, F5_s);
        const float F5_r02 = __fmaf_rn(F4_r02, F5_c, _v77);
        const float _v79 = __fmul_rn(F4_r10, F5_c);
        const float F5_r10 = __fmaf_rn((-F4_r12), F5_s, _v79);
        const float F5_r11 = F4_r11;
        const float _v81 = __fmul_rn(F4_r10, F5_s);
        const float F5_r12 = __fmaf_rn(F4_r12, F5_c, _v81);
        const float _v83 = __fmul_rn(F4_r20, F5_c);
        const float F5_r20 = __fmaf_rn((-F4_r22), F5_s, _v83);
        const float F5_r21 = F4_r21;
        const float _v85 = __fmul_rn(F4_r20, F5_s);
        const float F5_r22 = __fmaf_rn(F4_r22, F5_c, _v85);
        const float F5_t0 = _v72;
        const float F5_t1 = _v73;
        const float F5_t2 = _v74;
        const float _v87 = __fmaf_rn(1.0f, 0.0f, 0.0f);
        const float _v88 = __fmaf_rn(0.0f, 0.0f, _v87);
        const float s0_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v88);
        const float _v90 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v91 = __fmaf_rn(1.0f, 0.0f, _v90);
        const float s0_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v91);
        const float _v93 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v94 = __fmaf_rn(0.0f, 0.0f, _v93);
        const float s0_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v94);
        out[0] = s0_x; out[1] = s0_y; out[2] = s0_z; out[3] = 0.07999999821186066f;
        const float _v96 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v97 = __fmaf_rn(F0_r01, 0.0f, _v96);
        const float s1_x = __fmaf_rn(0.0f, 0.0f, _v97);
        const float _v99 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v100 = __fmaf_rn(F0_r11, 0.0f, _v99);
        const float s1_y = __fmaf_rn(0.0f, 0.0f, _v100);
        const float _v102 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
        const float _v103 = __fmaf_rn(0.0f, 0.0f, _v102);
        const float s1_z = __fmaf_rn(1.0f, 0.0f, _v103);
        out[4] = s1_x; out[5] = s1_y; out[6] = s1_z; out[7] = 0.07999999821186066f;
        const float _v105 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v106 = __fmaf_rn(F1_r01, 0.0f, _v105);
        const float s2_x = __fmaf_rn(F1_r02, 0.10499999672174454f, _v106);
        const float _v108 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v109 = __fmaf_rn(F1_r11, 0.0f, _v108);
        const float s2_y = __fmaf_rn(F1_r12, 0.10499999672174454f, _v109);
        const float _v111 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v112 = __fmaf_rn(0.0f, 0.0f, _v111);
        const float s2_z = __fmaf_rn(F1_r22, 0.10499999672174454f, _v112);
        out[8] = s2_x; out[9] = s2_y; out[10] = s2_z; out[11] = 0.07999999821186066f;
        const float _v114 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v115 = __fmaf_rn(F1_r01, 0.0f, _v114);
        const float s3_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v115);
        const float _v117 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v118 = __fmaf_rn(F1_r11, 0.0f, _v117);
        const float s3_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v118);
        const float _v120 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v121 = __fmaf_rn(0.0f, 0.0f, _v120);
        const float s3_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v121);
        out[12] = s3_x; out[13] = s3_y; out[14] = s3_z; out[15] = 0.07999999821186066f;
        const float _v123 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v124 = __fmaf_rn(F1_r01, 0.0f, _v123);
        const float s4_x = __fmaf_rn(F1_r02, 0.3149999976158142f, _v124);
        const float _v126 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v127 = __fmaf_rn(F1_r11, 0.0f, _v126);
        const float s4_y = __fmaf_rn(F1_r12, 0.3149999976158142f, _v127);
        const float _v129 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v130 = __fmaf_rn(0.0f, 0.0f, _v129);
        const float s4_z = __fmaf_rn(F1_r22, 0.3149999976158142f, _v130);
        out[16] = s4_x; out[17] = s4_y; out[18] = s4_z; out[19] = 0.07999999821186066f;
        const float _v132 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v133 = __fmaf_rn(F1_r01, 0.0f, _v132);
        const float s5_x = __fmaf_rn(F1_r02, 0.41999998688697815f, _v133);
        const float _v135 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v136 = __fmaf_rn(F1_r11, 0.0f, _v135);
        const float s5_y = __fmaf_rn(F1_r12, 0.41999998688697815f, _v136);
        const float _v138 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v139 = __fmaf_rn(0.0f, 0.0f, _v138);
        const float s5_z = __fmaf_rn(F1_r22, 0.41999998688697815f, _v139);
        out[20] = s5_x; out[21] = s5_y; out[22] = s5_z; out[23] = 0.07999999821186066f;
        const float _v141 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v142 = __fmaf_rn(F1_r01, 0.0f, _v141);
        const float s6_x = __fmaf_rn(F1_r02, 0.0f, _v142);
        const float _v144 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v145 = __fmaf_rn(F1_r11, 0.0f, _v144);
        const float s6_y = __fmaf_rn(F1_r12, 0.0f, _v145);
        const float _v147 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v148 = __fmaf_rn(0.0f, 0.0f, _v147);
        const float s6_z = __fmaf_rn(F1_r22, 0.0f, _v148);
        out[24] = s6_x; out[25] = s6_y; out[26] = s6_z; out[27] = 0.07999999821186066f;
        const float _v150 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v151 = __fmaf_rn(F2_r01, 0.0f, _v150);
        const float s7_x = __fmaf_rn(F2_r02, 0.0f, _v151);
        const float _v153 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v154 = __fmaf_rn(F2_r11, 0.0f, _v153);
        const float s7_y = __fmaf_rn(F2_r12, 0.0f, _v154);
        const float _v156 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v157 = __fmaf_rn(0.0f, 0.0f, _v156);
        const float s7_z = __fmaf_rn(F2_r22, 0.0f, _v157);
        out[28] = s7_x; out[29] = s7_y; out[30] = s7_z; out[31] = 0.07999999821186066f;
        const float _v159 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v160 = __fmaf_rn(F2_r01, 0.0f, _v159);
        const float s8_x = __fmaf_rn(F2_r02, 0.10000000149011612f, _v160);
        const float _v162 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v163 = __fmaf_rn(F2_r11, 0.0f, _v162);
        const float s8_y = __fmaf_rn(F2_r12, 0.10000000149011612f, _v163);
        const float _v165 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v166 = __fmaf_rn(0.0f, 0.0f, _v165);
        const float s8_z = __fmaf_rn(F2_r22, 0.10000000149011612f, _v166);
        out[32] = s8_x; out[33] = s8_y; out[34] = s8_z; out[35] = 0.03999999910593033f;
        const float _v168 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v169 = __fmaf_rn(F2_r01, 0.0f, _v168);
        const float s9_x = __fmaf_rn(F2_r02, 0.14000000059604645f, _v169);
        const float _v171 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v172 = __fmaf_rn(F2_r11, 0.0f, _v171);
        const float s9_y = __fmaf_rn(F2_r12, 0.14000000059604645f, _v172);
        const float _v174 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v175 = __fmaf_rn(0.0f, 0.0f, _v174);
        const float s9_z = __fmaf_rn(F2_r22, 0.14000000059604645f, _v175);
        out[36] = s9_x; out[37] = s9_y; out[38] = s9_z; out[39] = 0.03999999910593033f;
        const float _v177 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v178 = __fmaf_rn(F2_r01, 0.0f, _v177);
        const float s10_x = __fmaf_rn(F2_r02, 0.18000000715255737f, _v178);
        const float _v180 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v181 = __fmaf_rn(F2_r11, 0.0f, _v180);
        const float s10_y = __fmaf_rn(F2_r12, 0.18000000715255737f, _v181);
        const float _v183 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v184 = __fmaf_rn(0.0f, 0.0f, _v183);
        const float s10_z = __fmaf_rn(F2_r22, 0.18000000715255737f, _v184);
        out[40] = s10_x; out[41] = s10_y; out[42] = s10_z; out[43] = 0.03999999910593033f;
        const float _v186 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v187 = __fmaf_rn(F2_r01, 0.0f, _v186);
        const float s11_x = __fmaf_rn(F2_r02, 0.2199999988079071f, _v187);
        const float _v189 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v190 = __fmaf_rn(F2_r11, 0.0f, _v189);
        const float s11_y = __fmaf_rn(F2_r12, 0.2199999988079071f, _v190);
        const float _v192 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v193 = __fmaf_rn(0.0f, 0.0f, _v192);
        const float s11_z = __fmaf_rn(F2_r22, 0.2199999988079071f, _v193);
        out[44] = s11_x; out[45] = s11_y; out[46] = s11_z; out[47] = 0.03999999910593033f;
        const float _v195 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v196 = __fmaf_rn(F2_r01, 0.0f, _v195);
        const float s12_x = __fmaf_rn(F2_r02, 0.25999999046325684f, _v196);
        const float _v198 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v199 = __fmaf_rn(F2_r11, 0.0f, _v198);
        const float s12_y = __fmaf_rn(F2_r12, 0.25999999046325684f, _v199);
        const float _v201 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v202 = __fmaf_rn(0.0f, 0.0f, _v201);
        const float s12_z = __fmaf_rn(F2_r22, 0.25999999046325684f, _v202);
        out[48] = s12_x; out[49] = s12_y; out[50] = s12_z; out[51] = 0.03999999910593033f;
        const float _v204 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v205 = __fmaf_rn(F2_r01, 0.0f, _v204);
        const float s13_x = __fmaf_rn(F2_r02, 0.30000001192092896f, _v205);
        const float _v207 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v208 = __fmaf_rn(F2_r11, 0.0f, _v207);
        const float s13_y = __fmaf_rn(F2_r12, 0.30000001192092896f, _v208);
        const float _v210 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v211 = __fmaf_rn(0.0f, 0.0f, _v210);
        const float s13_z = __fmaf_rn(F2_r22, 0.30000001192092896f, _v211);
        out[52] = s13_x; out[53] = s13_y; out[54] = s13_z; out[55] = 0.03999999910593033f;
        const float _v213 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v214 = __fmaf_rn(F2_r01, 0.0f, _v213);
        const float s14_x = __fmaf_rn(F2_r02, 0.3400000035762787f, _v214);
        const float _v216 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v217 = __fmaf_rn(F2_r11, 0.0f, _v216);
        const float s14_y = __fmaf_rn(F2_r12, 0.3400000035762787f, _v217);
        const float _v219 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v220 = __fmaf_rn(0.0f, 0.0f, _v219);
        const float s14_z = __fmaf_rn(F2_r22, 0.3400000035762787f, _v220);
        out[56] = s14_x; out[57] = s14_y; out[58] = s14_z; out[59] = 0.03999999910593033f;
        const float _v222 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v223 = __fmaf_rn(F2_r01, 0.0f, _v222);
        const float s15_x = __fmaf_rn(F2_r02, 0.3799999952316284f, _v223);
        const float _v225 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v226 = __fmaf_rn(F2_r11, 0.0f, _v225);
        const float s15_y = __fmaf_rn(F2_r12, 0.3799999952316284f, _v226);
        const float _v228 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v229 = __fmaf_rn(0.0f, 0.0f, _v228);
        const float s15_z = __fmaf_rn(F2_r22, 0.3799999952316284f, _v229);
        out[60] = s15_x; out[61] = s15_y; out[62] = s15_z; out[63] = 0.03999999910593033f;
        const float _v231 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v232 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v231);
        const float s16_x = __fmaf_rn(F3_r02, 0.029999999329447746f, _v232);
        const float _v234 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v235 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v234);
        const float s16_y = __fmaf_rn(F3_r12, 0.029999999329447746f, _v235);
        const float _v237 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v238 = __fmaf_rn(0.0f, 0.09000000357627869f, _v237);
        const float s16_z = __fmaf_rn(F3_r22, 0.029999999329447746f, _v238);
        out[64] = s16_x; out[65] = s16_y; out[66] = s16_z; out[67] = 0.03999999910593033f;
        const float _v240 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v241 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v240);
        const float s17_x = __fmaf_rn(F3_r02, -0.029999999329447746f, _v241);
        const float _v243 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v244 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v243);
        const float s17_y = __fmaf_rn(F3_r12, -0.029999999329447746f, _v244);
        const float _v246 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v247 = __fmaf_rn(0.0f, 0.09000000357627869f, _v246);
        const float s17_z = __fmaf_rn(F3_r22, -0.029999999329447746f, _v247);
        out[68] = s17_x; out[69] = s17_y; out[70] = s17_z; out[71] = 0.03999999910593033f;
        const float _v249 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v250 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v249);
        const float s18_x = __fmaf_rn(F3_r02, 0.0f, _v250);
        const float _v252 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v253 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v252);
        const float s18_y = __fmaf_rn(F3_r12, 0.0f, _v253);
        const float _v255 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v256 = __fmaf_rn(0.0f, 0.09000000357627869f, _v255);
        const float s18_z = __fmaf_rn(F3_r22, 0.0f, _v256);
        out[72] = s18_x; out[73] = s18_y; out[74] = s18_z; out[75] = 0.03999999910593033f;
        const float _v258 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v259 = __fmaf_rn(F4_r01, 0.029999999329447746f, _v258);
        const float s19_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v259);
        const float _v261 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v262 = __fmaf_rn(F4_r11, 0.029999999329447746f, _v261);
        const float s19_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v262);
        const float _v264 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v265 = __fmaf_rn(F4_r21, 0.029999999329447746f, _v264);
        const float s19_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v265);
        out[76] = s19_x; out[77] = s19_y; out[78] = s19_z; out[79] = 0.03999999910593033f;
        const float _v267 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v268 = __fmaf_rn(F4_r01, -0.029999999329447746f, _v267);
        const float s20_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v268);
        const float _v270 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v271 = __fmaf_rn(F4_r11, -0.029999999329447746f, _v270);
        const float s20_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v271);
        const float _v273 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v274 = __fmaf_rn(F4_r21, -0.029999999329447746f, _v273);
        const float s20_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v274);
        out[80] = s20_x; out[81] = s20_y; out[82] = s20_z; out[83] = 0.03999999910593033f;
        const float _v276 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v277 = __fmaf_rn(F4_r01, 0.0f, _v276);
        const float s21_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v277);
        const float _v279 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v280 = __fmaf_rn(F4_r11, 0.0f, _v279);
        const float s21_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v280);
        const float _v282 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v283 = __fmaf_rn(F4_r21, 0.0f, _v282);
        const float s21_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v283);
        out[84] = s21_x; out[85] = s21_y; out[86] = s21_z; out[87] = 0.03999999910593033f;
        const float _v285 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
        const float _v286 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v285);
        const float s22_x = __fmaf_rn(F5_r02, 0.0f, _v286);
        const float _v288 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
        const float _v289 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v288);
        const float s22_y = __fmaf_rn(F5_r12, 0.0f, _v289);
        const float _v291 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
        const float _v292 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v291);
        const float s22_z = __fmaf_rn(F5_r22, 0.0f, _v292);
        out[88] = s22_x; out[89] = s22_y; out[90] = s22_z; out[91] = 0.03999999910593033f;
        const float _v294 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
        const float _v295 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v294);
        const float s23_x = __fmaf_rn(F5_r02, 0.0f, _v295);
        const float _v297 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
        const float _v298 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v297);
        const float s23_y = __fmaf_rn(F5_r12, 0.0f, _v298);
        const float _v300 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
        const float _v301 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v300);
        const float s23_z = __fmaf_rn(F5_r22, 0.0f, _v301);
        out[92] = s23_x; out[93] = s23_y; out[94] = s23_z; out[95] = 0.03999999910593033f;
        const float _v303 = __fmaf_rn(F5_r00, -4.7779416490811855e-05f, F5_t0);
        const float _v304 = __fmaf_rn(F5_r01, 0.17729996144771576f, _v303);
        const float s24_x = __fmaf_rn(F5_r02, 0.0005477796075865626f, _v304);
        const float _v306 = __fmaf_rn(F5_r10, -4.7779416490811855e-05f, F5_t1);
        const float _v307 = __fmaf_rn(F5_r11, 0.17729996144771576f, _v306);
        const float s24_y = __fmaf_rn(F5_r12, 0.0005477796075865626f, _v307);
        const float _v309 = __fmaf_rn(F5_r20, -4.7779416490811855e-05f, F5_t2);
        const float _v310 = __fmaf_rn(F5_r21, 0.17729996144771576f, _v309);
        const float s24_z = __fmaf_rn(F5_r22, 0.0005477796075865626f, _v310);
        out[96] = s24_x; out[97] = s24_y; out[98] = s24_z; out[99] = 0.03999999910593033f;
        const float _v312 = __fmaf_rn(F5_r00, -1.592643093317747e-05f, F5_t0);
        const float _v313 = __fmaf_rn(F5_r01, 0.13729998469352722f, _v312);
        const float s25_x = __fmaf_rn(F5_r02, 0.000515926512889564f, _v313);
        const float _v315 = __fmaf_rn(F5_r10, -1.592643093317747e-05f, F5_t1);
        const float _v316 = __fmaf_rn(F5_r11, 0.13729998469352722f, _v315);
        const float s25_y = __fmaf_rn(F5_r12, 0.000515926512889564f, _v316);
        const float _v318 = __fmaf_rn(F5_r20, -1.592643093317747e-05f, F5_t2);
        const float _v319 = __fmaf_rn(F5_r21, 0.13729998469352722f, _v318);
        const float s25_z = __fmaf_rn(F5_r22, 0.000515926512889564f, _v319);
        out[100] = s25_x; out[101] = s25_y; out[102] = s25_z; out[103] = 0.03999999910593033f;
        const float _v321 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
        const float _v322 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v321);
        const float s26_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v322);
        const float _v324 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
        const float _v325 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v324);
        const float s26_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v325);
        const float _v327 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
        const float _v328 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v327);
        const float s26_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v328);
        out[104] = s26_x; out[105] = s26_y; out[106] = s26_z; out[107] = 0.019999999552965164f;
        const float _v330 = __fmaf_rn(F5_r00, 0.047173965722322464f, F5_t0);
        const float _v331 = __fmaf_rn(F5_r01, 0.2571420967578888f, _v330);
        const float s27_x = __fmaf_rn(F5_r02, 0.0006113300914876163f, _v331);
        const float _v333 = __fmaf_rn(F5_r10, 0.047173965722322464f, F5_t1);
        const float _v334 = __fmaf_rn(F5_r11, 0.2571420967578888f, _v333);
        const float s27_y = __fmaf_rn(F5_r12, 0.0006113300914876163f, _v334);
        const float _v336 = __fmaf_rn(F5_r20, 0.047173965722322464f, F5_t2);
        const float _v337 = __fmaf_rn(F5_r21, 0.2571420967578888f, _v336);
        const float s27_z = __fmaf_rn(F5_r22, 0.0006113300914876163f, _v337);
        out[108] = s27_x; out[109] = s27_y; out[110] = s27_z; out[111] = 0.014999999664723873f;
        const float _v339 = __fmaf_rn(F5_r00, 0.047193873673677444f, F5_t0);
        const float _v340 = __fmaf_rn(F5_r01, 0.2321421056985855f, _v339);
        const float s28_x = __fmaf_rn(F5_r02, 0.0005914219073019922f, _v340);
        const float _v342 = __fmaf_rn(F5_r10, 0.047193873673677444f, F5_t1);
        const float _v343 = __fmaf_rn(F5_r11, 0.2321421056985855f, _v342);
        const float s28_y = __fmaf_rn(F5_r12, 0.0005914219073019922f, _v343);
        const float _v345 = __fmaf_rn(F5_r20, 0.047193873673677444f, F5_t2);
        const float _v346 = __fmaf_rn(F5_r21, 0.2321421056985855f, _v345);
        const float s28_z = __fmaf_rn(F5_r22, 0.0005914219073019922f, _v346);
        out[112] = s28_x; out[113] = s28_y; out[114] = s28_z; out[115] = 0.014999999664723873f;
        const float _v348 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
        const float _v349 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v348);
        const float s29_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v349);
        const float _v351 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
        const float _v352 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v351);
        const float s29_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v352);
        const float _v354 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
        const float _v355 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v354);
        const float s29_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v355);
        out[116] = s29_x; out[117] = s29_y; out[118] = s29_z; out[119] = 0.019999999552965164f;
        const float _v357 = __fmaf_rn(F5_r00, 0.06221185252070427f, F5_t0);
        const float _v358 = __fmaf_rn(F5_r01, 0.21820759773254395f, _v357);
        const float s30_x = __fmaf_rn(F5_r02, 0.0005803159438073635f, _v358);
        const float _v360 = __fmaf_rn(F5_r10, 0.06221185252070427f, F5_t1);
        const float _v361 = __fmaf_rn(F5_r11, 0.21820759773254395f, _v360);
        const float s30_y = __fmaf_rn(F5_r12, 0.0005803159438073635f, _v361);
        const float _v363 = __fmaf_rn(F5_r20, 0.06221185252070427f, F5_t2);
        const float _v364 = __fmaf_rn(F5_r21, 0.21820759773254395f, _v363);
        const float s30_z = __fmaf_rn(F5_r22, 0.0005803159438073635f, _v364);
        out[120] = s30_x; out[121] = s30_y; out[122] = s30_z; out[123] = 0.014999999664723873f;
        const float _v366 = __fmaf_rn(F5_r00, 0.06224370747804642f, F5_t0);
        const float _v367 = __fmaf_rn(F5_r01, 0.1782076209783554f, _v366);
        const float s31_x = __fmaf_rn(F5_r02, 0.0005484629073180258f, _v367);
        const float _v369 = __fmaf_rn(F5_r10, 0.06224370747804642f, F5_t1);
        const float _v370 = __fmaf_rn(F5_r11, 0.1782076209783554f, _v369);
        const float s31_y = __fmaf_rn(F5_r12, 0.0005484629073180258f, _v370);
        const float _v372 = __fmaf_rn(F5_r20, 0.06224370747804642f, F5_t2);
        const float _v373 = __fmaf_rn(F5_r21, 0.1782076209783554f, _v372);
        const float s31_z = __fmaf_rn(F5_r22, 0.0005484629073180258f, _v373);
        out[124] = s31_x; out[125] = s31_y; out[126] = s31_z; out[127] = 0.014999999664723873f;
        const float _v375 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
        const float _v376 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v375);
        const float s32_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v376);
        const float _v378 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
        const float _v379 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v378);
        const float s32_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v379);
        const float _v381 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
        const float _v382 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v381);
        const float s32_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v382);
        out[128] = s32_x; out[129] = s32_y; out[130] = s32_z; out[131] = 0.014999999664723873f;
        const float _v384 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
        const float _v385 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v384);
        const float s33_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v385);
        const float _v387 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
        const float _v388 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v387);
        const float s33_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v388);
        const float _v390 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
        const float _v391 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v390);
        const float s33_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v391);
        out[132] = s33_x; out[133] = s33_y; out[134] = s33_z; out[135] = 0.019999999552965164f;
        const float _v393 = __fmaf_rn(F5_r00, -0.04691765084862709f, F5_t0);
        const float _v394 = __fmaf_rn(F5_r01, 0.25742751359939575f, _v393);
        const float s34_x = __fmaf_rn(F5_r02, 0.0006116170552559197f, _v394);
        const float _v396 = __fmaf_rn(F5_r10, -0.04691765084862709f, F5_t1);
        const float _v397 = __fmaf_rn(F5_r11, 0.25742751359939575f, _v396);
        const float s34_y = __fmaf_rn(F5_r12, 0.0006116170552559197f, _v397);
        const float _v399 = __fmaf_rn(F5_r20, -0.04691765084862709f, F5_t2);
        const float _v400 = __fmaf_rn(F5_r21, 0.25742751359939575f, _v399);
        const float s34_z = __fmaf_rn(F5_r22, 0.0006116170552559197f, _v400);
        out[136] = s34_x; out[137] = s34_y; out[138] = s34_z; out[139] = 0.014999999664723873f;
        const float _v402 = __fmaf_rn(F5_r00, -0.04689774289727211f, F5_t0);
        const float _v403 = __fmaf_rn(F5_r01, 0.23242753744125366f, _v402);
        const float s35_x = __fmaf_rn(F5_r02, 0.0005917088710702956f, _v403);
        const float _v405 = __fmaf_rn(F5_r10, -0.04689774289727211f, F5_t1);
        const float _v406 = __fmaf_rn(F5_r11, 0.23242753744125366f, _v405);
        const float s35_y = __fmaf_rn(F5_r12, 0.0005917088710702956f, _v406);
        const float _v408 = __fmaf_rn(F5_r20, -0.04689774289727211f, F5_t2);
        const float _v409 = __fmaf_rn(F5_r21, 0.23242753744125366f, _v408);
        const float s35_z = __fmaf_rn(F5_r22, 0.0005917088710702956f, _v409);
        out[140] = s35_x; out[141] = s35_y; out[142] = s35_z; out[143] = 0.014999999664723873f;
        const float _v411 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
        const float _v412 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v411);
        const float s36_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v412);
        const float _v414 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
        const float _v415 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v414);
        const float s36_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v415);
        const float _v417 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
        const float _v418 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v417);
        const float s36_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v418);
        out[144] = s36_x; out[145] = s36_y; out[146] = s36_z; out[147] = 0.019999999552965164f;
        const float _v420 = __fmaf_rn(F5_r00, -0.06239129602909088f, F5_t0);
        const float _v421 = __fmaf_rn(F5_r01, 0.218440979719162f, _v420);
        const float s37_x = __fmaf_rn(F5_r02, 0.0005805808468721807f, _v421);
        const float _v423 = __fmaf_rn(F5_r10, -0.06239129602909088f, F5_t1);
        const float _v424 = __fmaf_rn(F5_r11, 0.218440979719162f, _v423);
        const float s37_y = __fmaf_rn(F5_r12, 0.0005805808468721807f, _v424);
        const float _v426 = __fmaf_rn(F5_r20, -0.06239129602909088f, F5_t2);
        const float _v427 = __fmaf_rn(F5_r21, 0.218440979719162f, _v426);
        const float s37_z = __fmaf_rn(F5_r22, 0.0005805808468721807f, _v427);
        out[148] = s37_x; out[149] = s37_y; out[150] = s37_z; out[151] = 0.014999999664723873f;
        const float _v429 = __fmaf_rn(F5_r00, -0.06235944479703903f, F5_t0);
        const float _v430 = __fmaf_rn(F5_r01, 0.17844100296497345f, _v429);
        const float s38_x = __fmaf_rn(F5_r02, 0.0005487277521751821f, _v430);
        const float _v432 = __fmaf_rn(F5_r10, -0.06235944479703903f, F5_t1);
        const float _v433 = __fmaf_rn(F5_r11, 0.17844100296497345f, _v432);
        const float s38_y = __fmaf_rn(F5_r12, 0.0005487277521751821f, _v433);
        const float _v435 = __fmaf_rn(F5_r20, -0.06235944479703903f, F5_t2);
        const float _v436 = __fmaf_rn(F5_r21, 0.17844100296497345f, _v435);
        const float s38_z = __fmaf_rn(F5_r22, 0.0005487277521751821f, _v436);
        out[152] = s38_x; out[153] = s38_y; out[154] = s38_z; out[155] = 0.014999999664723873f;
        const float _v438 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
        const float _v439 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v438);
        const float s39_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v439);
        const float _v441 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
        const float _v442 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v441);
        const float s39_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v442);
        const float _v444 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
        const float _v445 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v444);
        const float s39_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v445);
        out[156] = s39_x; out[157] = s39_y; out[158] = s39_z; out[159] = 0.014999999664723873f;
        const float _v447 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
        const float _v448 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v447);
        const float s40_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v448);
        const float _v450 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
        const float _v451 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v450);
        const float s40_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v451);
        const float _v453 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
        const float _v454 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v453);
        const float s40_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v454);
        out[160] = s40_x; out[161] = s40_y; out[162] = s40_z; out[163] = 0.03500000014901161f;
        const float _v456 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
        const float _v457 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v456);
        const float s41_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v457);
        const float _v459 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
        const float _v460 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v459);
        const float s41_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v460);
        const float _v462 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
        const float _v463 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v462);
        const float s41_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v463);
        out[164] = s41_x; out[165] = s41_y; out[166] = s41_z; out[167] = 0.019999999552965164f;
        const float _v465 = __fmaf_rn(F5_r00, -0.0469076968729496f, F5_t0);
        const float _v466 = __fmaf_rn(F5_r01, 0.2449275404214859f, _v465);
        const float s42_x = __fmaf_rn(F5_r02, 0.0006016629631631076f, _v466);
        const float _v468 = __fmaf_rn(F5_r10, -0.0469076968729496f, F5_t1);
        const float _v469 = __fmaf_rn(F5_r11, 0.2449275404214859f, _v468);
        const float s42_y = __fmaf_rn(F5_r12, 0.0006016629631631076f, _v469);
        const float _v471 = __fmaf_rn(F5_r20, -0.0469076968729496f, F5_t2);
        const float _v472 = __fmaf_rn(F5_r21, 0.2449275404214859f, _v471);
        const float s42_z = __fmaf_rn(F5_r22, 0.0006016629631631076f, _v472);
        out[168] = s42_x; out[169] = s42_y; out[170] = s42_z; out[171] = 0.027499999850988388f;
        const float _v474 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
        const float _v475 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v474);
        const float s43_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v475);
        const float _v477 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
        const float _v478 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v477);
        const float s43_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v478);
        const float _v480 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
        const float _v481 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v480);
        const float s43_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v481);
        out[172] = s43_x; out[173] = s43_y; out[174] = s43_z; out[175] = 0.019999999552965164f;
        const float _v483 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
        const float _v484 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v483);
        const float s44_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v484);
        const float _v486 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
        const float _v487 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v486);
        const float s44_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v487);
        const float _v489 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
        const float _v490 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v489);
        const float s44_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v490);
        out[176] = s44_x; out[177] = s44_y; out[178] = s44_z; out[179] = 0.03500000014901161f;
        const float _v492 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
        const float _v493 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v492);
        const float s45_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v493);
        const float _v495 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
        const float _v496 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v495);
        const float s45_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v496);
        const float _v498 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
        const float _v499 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v498);
        const float s45_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v499);
        out[180] = s45_x; out[181] = s45_y; out[182] = s45_z; out[183] = 0.019999999552965164f;
        const float _v501 = __fmaf_rn(F5_r00, 0.047183919697999954f, F5_t0);
        const float _v502 = __fmaf_rn(F5_r01, 0.24464209377765656f, _v501);
        const float s46_x = __fmaf_rn(F5_r02, 0.0006013759993948042f, _v502);
        const float _v504 = __fmaf_rn(F5_r10, 0.047183919697999954f, F5_t1);
        const float _v505 = __fmaf_rn(F5_r11, 0.24464209377765656f, _v504);
        const float s46_y = __fmaf_rn(F5_r12, 0.0006013759993948042f, _v505);
        const float _v507 = __fmaf_rn(F5_r20, 0.047183919697999954f, F5_t2);
        const float _v508 = __fmaf_rn(F5_r21, 0.24464209377765656f, _v507);
        const float s46_z = __fmaf_rn(F5_r22, 0.0006013759993948042f, _v508);
        out[184] = s46_x; out[185] = s46_y; out[186] = s46_z; out[187] = 0.027499999850988388f;
        const float _v510 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
        const float _v511 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v510);
        const float s47_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v511);
        const float _v513 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
        const float _v514 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v513);
        const float s47_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v514);
        const float _v516 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
        const float _v517 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v516);
        const float s47_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v517);
        out[188] = s47_x; out[189] = s47_y; out[190] = s47_z; out[191] = 0.019999999552965164f;
        const float _v519 = __fmaf_rn(F5_r00, -3.185292371199466e-05f, F5_t0);
        const float _v520 = __fmaf_rn(F5_r01, 0.1572999805212021f, _v519);
        const float s48_x = __fmaf_rn(F5_r02, 0.0005318530602380633f, _v520);
        const float _v522 = __fmaf_rn(F5_r10, -3.185292371199466e-05f, F5_t1);
        const float _v523 = __fmaf_rn(F5_r11, 0.1572999805212021f, _v522);
        const float s48_y = __fmaf_rn(F5_r12, 0.0005318530602380633f, _v523);
        const float _v525 = __fmaf_rn(F5_r20, -3.185292371199466e-05f, F5_t2);
        const float _v526 = __fmaf_rn(F5_r21, 0.1572999805212021f, _v525);
        const float s48_z = __fmaf_rn(F5_r22, 0.0005318530602380633f, _v526);
        out[192] = s48_x; out[193] = s48_y; out[194] = s48_z; out[195] = 0.05999999865889549f;
        const float _v528 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
        const float _v529 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v528);
        const float s49_x = __fmaf_rn(F5_r02, 0.0f, _v529);
        const float _v531 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
        const float _v532 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v531);
        const float s49_y = __fmaf_rn(F5_r12, 0.0f, _v532);
        const float _v534 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
        const float _v535 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v534);
        const float s49_z = __fmaf_rn(F5_r22, 0.0f, _v535);
        out[196] = s49_x; out[197] = s49_y; out[198] = s49_z; out[199] = 0.03999999910593033f;
        const float _v537 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
        const float _v538 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v537);
        const float s50_x = __fmaf_rn(F5_r02, 0.0f, _v538);
        const float _v540 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
        const float _v541 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v540);
        const float s50_y = __fmaf_rn(F5_r12, 0.0f, _v541);
        const float _v543 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
        const float _v544 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v543);
        const float s50_z = __fmaf_rn(F5_r22, 0.0f, _v544);
        out[200] = s50_x; out[201] = s50_y; out[202] = s50_z; out[203] = 0.03999999910593033f;
        const float _v546 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v547 = __fmaf_rn(F4_r01, 0.0f, _v546);
        const float s51_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v547);
        const float _v549 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v550 = __fmaf_rn(F4_r11, 0.0f, _v549);
        const float s51_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v550);
        const float _v552 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v553 = __fmaf_rn(F4_r21, 0.0f, _v552);
        const float s51_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v553);
        out[204] = s51_x; out[205] = s51_y; out[206] = s51_z; out[207] = 0.07000000029802322f;
        const float _v555 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v556 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v555);
        const float s52_x = __fmaf_rn(F3_r02, 0.0f, _v556);
        const float _v558 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v559 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v558);
        const float s52_y = __fmaf_rn(F3_r12, 0.0f, _v559);
        const float _v561 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v562 = __fmaf_rn(0.0f, 0.09000000357627869f, _v561);
        const float s52_z = __fmaf_rn(F3_r22, 0.0f, _v562);
        out[208] = s52_x; out[209] = s52_y; out[210] = s52_z; out[211] = 0.07000000029802322f;
        const float _v564 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v565 = __fmaf_rn(F2_r01, 0.0f, _v564);
        const float s53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v565);
        const float _v567 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v568 = __fmaf_rn(F2_r11, 0.0f, _v567);
        const float s53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v568);
        const float _v570 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v571 = __fmaf_rn(0.0f, 0.0f, _v570);
        const float s53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v571);
        out[212] = s53_x; out[213] = s53_y; out[214] = s53_z; out[215] = 0.25f;
        const float _v573 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v574 = __fmaf_rn(F1_r01, 0.0f, _v573);
        const float s54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v574);
        const float _v576 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v577 = __fmaf_rn(F1_r11, 0.0f, _v576);
        const float s54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v577);
        const float _v579 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v580 = __fmaf_rn(0.0f, 0.0f, _v579);
        const float s54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v580);
        out[216] = s54_x; out[217] = s54_y; out[218] = s54_z; out[219] = 0.28999999165534973f;
        const float _v582 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v583 = __fmaf_rn(F0_r01, 0.0f, _v582);
        const float s55_x = __fmaf_rn(0.0f, 0.0f, _v583);
        const float _v585 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v586 = __fmaf_rn(F0_r11, 0.0f, _v585);
        const float s55_y = __fmaf_rn(0.0f, 0.0f, _v586);
        const float _v588 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
        const float _v589 = __fmaf_rn(0.0f, 0.0f, _v588);
        const float s55_z = __fmaf_rn(1.0f, 0.0f, _v589);
        out[220] = s55_x; out[221] = s55_y; out[222] = s55_z; out[223] = 0.07999999821186066f;
        const float _v591 = __fmaf_rn(1.0f, 0.0f, 0.0f);
        const float _v592 = __fmaf_rn(0.0f, 0.0f, _v591);
        const float s56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v592);
        const float _v594 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v595 = __fmaf_rn(1.0f, 0.0f, _v594);
        const float s56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v595);
        const float _v597 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v598 = __fmaf_rn(0.0f, 0.0f, _v597);
        const float s56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v598);
        out[224] = s56_x; out[225] = s56_y; out[226] = s56_z; out[227] = 0.07999999821186066f;
    }

    // fine spheres [37, 38, 39] (robotiq_85_right_finger_link)
    static __device__ __noinline__ void fine_0(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, -0.06239129602909088f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.218440979719162f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005805808468721807f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, -0.06239129602909088f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.218440979719162f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005805808468721807f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, -0.06239129602909088f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.218440979719162f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005805808468721807f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.014999999664723873f);
        const float _v100009 = __fmaf_rn(F5_r00, -0.06235944479703903f, F5_t0);
        const float _v100010 = __fmaf_rn(F5_r01, 0.17844100296497345f, _v100009);
        const float s1_x = __fmaf_rn(F5_r02, 0.0005487277521751821f, _v100010);
        const float _v100012 = __fmaf_rn(F5_r10, -0.06235944479703903f, F5_t1);
        const float _v100013 = __fmaf_rn(F5_r11, 0.17844100296497345f, _v100012);
        const float s1_y = __fmaf_rn(F5_r12, 0.0005487277521751821f, _v100013);
        const float _v100015 = __fmaf_rn(F5_r20, -0.06235944479703903f, F5_t2);
        const float _v100016 = __fmaf_rn(F5_r21, 0.17844100296497345f, _v100015);
        const float s1_z = __fmaf_rn(F5_r22, 0.0005487277521751821f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.014999999664723873f);
        const float _v100018 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
        const float _v100019 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v100018);
        const float s2_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v100019);
        const float _v100021 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
        const float _v100022 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v100021);
        const float s2_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v100022);
        const float _v100024 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
        const float _v100025 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v100024);
        const float s2_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.014999999664723873f);
    }
    // fine spheres [36] (robotiq_85_right_knuckle_link)
    static __device__ __noinline__ void fine_1(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.019999999552965164f);
    }
    // fine spheres [34, 35] (robotiq_85_right_finger_tip_link)
    static __device__ __noinline__ void fine_2(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, -0.04691765084862709f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.25742751359939575f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0006116170552559197f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, -0.04691765084862709f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.25742751359939575f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0006116170552559197f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, -0.04691765084862709f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.25742751359939575f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0006116170552559197f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.014999999664723873f);
        const float _v100009 = __fmaf_rn(F5_r00, -0.04689774289727211f, F5_t0);
        const float _v100010 = __fmaf_rn(F5_r01, 0.23242753744125366f, _v100009);
        const float s1_x = __fmaf_rn(F5_r02, 0.0005917088710702956f, _v100010);
        const float _v100012 = __fmaf_rn(F5_r10, -0.04689774289727211f, F5_t1);
        const float _v100013 = __fmaf_rn(F5_r11, 0.23242753744125366f, _v100012);
        const float s1_y = __fmaf_rn(F5_r12, 0.0005917088710702956f, _v100013);
        const float _v100015 = __fmaf_rn(F5_r20, -0.04689774289727211f, F5_t2);
        const float _v100016 = __fmaf_rn(F5_r21, 0.23242753744125366f, _v100015);
        const float s1_z = __fmaf_rn(F5_r22, 0.0005917088710702956f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.014999999664723873f);
    }
    // fine spheres [33] (robotiq_85_right_inner_knuckle_link)
    static __device__ __noinline__ void fine_3(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.019999999552965164f);
    }
    // fine spheres [30, 31, 32] (robotiq_85_left_finger_link)
    static __device__ __noinline__ void fine_4(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 0.06221185252070427f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.21820759773254395f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005803159438073635f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 0.06221185252070427f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.21820759773254395f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005803159438073635f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 0.06221185252070427f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.21820759773254395f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005803159438073635f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.014999999664723873f);
        const float _v100009 = __fmaf_rn(F5_r00, 0.06224370747804642f, F5_t0);
        const float _v100010 = __fmaf_rn(F5_r01, 0.1782076209783554f, _v100009);
        const float s1_x = __fmaf_rn(F5_r02, 0.0005484629073180258f, _v100010);
        const float _v100012 = __fmaf_rn(F5_r10, 0.06224370747804642f, F5_t1);
        const float _v100013 = __fmaf_rn(F5_r11, 0.1782076209783554f, _v100012);
        const float s1_y = __fmaf_rn(F5_r12, 0.0005484629073180258f, _v100013);
        const float _v100015 = __fmaf_rn(F5_r20, 0.06224370747804642f, F5_t2);
        const float _v100016 = __fmaf_rn(F5_r21, 0.1782076209783554f, _v100015);
        const float s1_z = __fmaf_rn(F5_r22, 0.0005484629073180258f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.014999999664723873f);
        const float _v100018 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
        const float _v100019 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v100018);
        const float s2_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v100019);
        const float _v100021 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
        const float _v100022 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v100021);
        const float s2_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v100022);
        const float _v100024 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
        const float _v100025 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v100024);
        const float s2_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.014999999664723873f);
    }
    // fine spheres [29] (robotiq_85_left_knuckle_link)
    static __device__ __noinline__ void fine_5(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.019999999552965164f);
    }
    // fine spheres [27, 28] (robotiq_85_left_finger_tip_link)
    static __device__ __noinline__ void fine_6(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 0.047173965722322464f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.2571420967578888f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0006113300914876163f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 0.047173965722322464f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.2571420967578888f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0006113300914876163f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 0.047173965722322464f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.2571420967578888f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0006113300914876163f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.014999999664723873f);
        const float _v100009 = __fmaf_rn(F5_r00, 0.047193873673677444f, F5_t0);
        const float _v100010 = __fmaf_rn(F5_r01, 0.2321421056985855f, _v100009);
        const float s1_x = __fmaf_rn(F5_r02, 0.0005914219073019922f, _v100010);
        const float _v100012 = __fmaf_rn(F5_r10, 0.047193873673677444f, F5_t1);
        const float _v100013 = __fmaf_rn(F5_r11, 0.2321421056985855f, _v100012);
        const float s1_y = __fmaf_rn(F5_r12, 0.0005914219073019922f, _v100013);
        const float _v100015 = __fmaf_rn(F5_r20, 0.047193873673677444f, F5_t2);
        const float _v100016 = __fmaf_rn(F5_r21, 0.2321421056985855f, _v100015);
        const float s1_z = __fmaf_rn(F5_r22, 0.0005914219073019922f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.014999999664723873f);
    }
    // fine spheres [26] (robotiq_85_left_inner_knuckle_link)
    static __device__ __noinline__ void fine_7(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.019999999552965164f);
    }
    // fine spheres [24, 25] (robotiq_85_base_link)
    static __device__ __noinline__ void fine_8(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, -4.7779416490811855e-05f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.17729996144771576f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0005477796075865626f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, -4.7779416490811855e-05f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.17729996144771576f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0005477796075865626f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, -4.7779416490811855e-05f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.17729996144771576f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0005477796075865626f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.03999999910593033f);
        const float _v100009 = __fmaf_rn(F5_r00, -1.592643093317747e-05f, F5_t0);
        const float _v100010 = __fmaf_rn(F5_r01, 0.13729998469352722f, _v100009);
        const float s1_x = __fmaf_rn(F5_r02, 0.000515926512889564f, _v100010);
        const float _v100012 = __fmaf_rn(F5_r10, -1.592643093317747e-05f, F5_t1);
        const float _v100013 = __fmaf_rn(F5_r11, 0.13729998469352722f, _v100012);
        const float s1_y = __fmaf_rn(F5_r12, 0.000515926512889564f, _v100013);
        const float _v100015 = __fmaf_rn(F5_r20, -1.592643093317747e-05f, F5_t2);
        const float _v100016 = __fmaf_rn(F5_r21, 0.13729998469352722f, _v100015);
        const float s1_z = __fmaf_rn(F5_r22, 0.000515926512889564f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.03999999910593033f);
    }
    // fine spheres [23] (fts_robotside)
    static __device__ __noinline__ void fine_9(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.03999999910593033f);
    }
    // fine spheres [22] (wrist_3_link)
    static __device__ __noinline__ void fine_10(const float F5_r00, const float F5_r01, const float F5_r02, const float F5_r10, const float F5_r11, const float F5_r12, const float F5_r20, const float F5_r21, const float F5_r22, const float F5_t0, const float F5_t1, const float F5_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
        const float _v100001 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v100000);
        const float s0_x = __fmaf_rn(F5_r02, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
        const float _v100004 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v100003);
        const float s0_y = __fmaf_rn(F5_r12, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
        const float _v100007 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v100006);
        const float s0_z = __fmaf_rn(F5_r22, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.03999999910593033f);
    }
    // fine spheres [19, 20, 21] (wrist_2_link)
    static __device__ __noinline__ void fine_11(const float F4_r00, const float F4_r01, const float F4_r02, const float F4_r10, const float F4_r11, const float F4_r12, const float F4_r20, const float F4_r21, const float F4_r22, const float F4_t0, const float F4_t1, const float F4_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100001 = __fmaf_rn(F4_r01, 0.029999999329447746f, _v100000);
        const float s0_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v100001);
        const float _v100003 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100004 = __fmaf_rn(F4_r11, 0.029999999329447746f, _v100003);
        const float s0_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v100004);
        const float _v100006 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100007 = __fmaf_rn(F4_r21, 0.029999999329447746f, _v100006);
        const float s0_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.03999999910593033f);
        const float _v100009 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100010 = __fmaf_rn(F4_r01, -0.029999999329447746f, _v100009);
        const float s1_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v100010);
        const float _v100012 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100013 = __fmaf_rn(F4_r11, -0.029999999329447746f, _v100012);
        const float s1_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v100013);
        const float _v100015 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100016 = __fmaf_rn(F4_r21, -0.029999999329447746f, _v100015);
        const float s1_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.03999999910593033f);
        const float _v100018 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
        const float _v100019 = __fmaf_rn(F4_r01, 0.0f, _v100018);
        const float s2_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v100019);
        const float _v100021 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
        const float _v100022 = __fmaf_rn(F4_r11, 0.0f, _v100021);
        const float s2_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v100022);
        const float _v100024 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
        const float _v100025 = __fmaf_rn(F4_r21, 0.0f, _v100024);
        const float s2_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.03999999910593033f);
    }
    // fine spheres [16, 17, 18] (wrist_1_link)
    static __device__ __noinline__ void fine_12(const float F3_r00, const float F3_r01, const float F3_r02, const float F3_r10, const float F3_r11, const float F3_r12, const float F3_r20, const float F3_r22, const float F3_t0, const float F3_t1, const float F3_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v100001 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v100000);
        const float s0_x = __fmaf_rn(F3_r02, 0.029999999329447746f, _v100001);
        const float _v100003 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v100004 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v100003);
        const float s0_y = __fmaf_rn(F3_r12, 0.029999999329447746f, _v100004);
        const float _v100006 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v100007 = __fmaf_rn(0.0f, 0.09000000357627869f, _v100006);
        const float s0_z = __fmaf_rn(F3_r22, 0.029999999329447746f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.03999999910593033f);
        const float _v100009 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v100010 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v100009);
        const float s1_x = __fmaf_rn(F3_r02, -0.029999999329447746f, _v100010);
        const float _v100012 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v100013 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v100012);
        const float s1_y = __fmaf_rn(F3_r12, -0.029999999329447746f, _v100013);
        const float _v100015 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v100016 = __fmaf_rn(0.0f, 0.09000000357627869f, _v100015);
        const float s1_z = __fmaf_rn(F3_r22, -0.029999999329447746f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.03999999910593033f);
        const float _v100018 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
        const float _v100019 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v100018);
        const float s2_x = __fmaf_rn(F3_r02, 0.0f, _v100019);
        const float _v100021 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
        const float _v100022 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v100021);
        const float s2_y = __fmaf_rn(F3_r12, 0.0f, _v100022);
        const float _v100024 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
        const float _v100025 = __fmaf_rn(0.0f, 0.09000000357627869f, _v100024);
        const float s2_z = __fmaf_rn(F3_r22, 0.0f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.03999999910593033f);
    }
    // fine spheres [7, 8, 9, 10, 11, 12, 13, 14, 15] (forearm_link)
    static __device__ __noinline__ void fine_13(const float F2_r00, const float F2_r01, const float F2_r02, const float F2_r10, const float F2_r11, const float F2_r12, const float F2_r20, const float F2_r22, const float F2_t0, const float F2_t1, const float F2_t2, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100001 = __fmaf_rn(F2_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(F2_r02, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100004 = __fmaf_rn(F2_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(F2_r12, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100007 = __fmaf_rn(0.0f, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(F2_r22, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.07999999821186066f);
        const float _v100009 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100010 = __fmaf_rn(F2_r01, 0.0f, _v100009);
        const float s1_x = __fmaf_rn(F2_r02, 0.10000000149011612f, _v100010);
        const float _v100012 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100013 = __fmaf_rn(F2_r11, 0.0f, _v100012);
        const float s1_y = __fmaf_rn(F2_r12, 0.10000000149011612f, _v100013);
        const float _v100015 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100016 = __fmaf_rn(0.0f, 0.0f, _v100015);
        const float s1_z = __fmaf_rn(F2_r22, 0.10000000149011612f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.03999999910593033f);
        const float _v100018 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100019 = __fmaf_rn(F2_r01, 0.0f, _v100018);
        const float s2_x = __fmaf_rn(F2_r02, 0.14000000059604645f, _v100019);
        const float _v100021 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100022 = __fmaf_rn(F2_r11, 0.0f, _v100021);
        const float s2_y = __fmaf_rn(F2_r12, 0.14000000059604645f, _v100022);
        const float _v100024 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100025 = __fmaf_rn(0.0f, 0.0f, _v100024);
        const float s2_z = __fmaf_rn(F2_r22, 0.14000000059604645f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.03999999910593033f);
        const float _v100027 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100028 = __fmaf_rn(F2_r01, 0.0f, _v100027);
        const float s3_x = __fmaf_rn(F2_r02, 0.18000000715255737f, _v100028);
        const float _v100030 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100031 = __fmaf_rn(F2_r11, 0.0f, _v100030);
        const float s3_y = __fmaf_rn(F2_r12, 0.18000000715255737f, _v100031);
        const float _v100033 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100034 = __fmaf_rn(0.0f, 0.0f, _v100033);
        const float s3_z = __fmaf_rn(F2_r22, 0.18000000715255737f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.03999999910593033f);
        const float _v100036 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100037 = __fmaf_rn(F2_r01, 0.0f, _v100036);
        const float s4_x = __fmaf_rn(F2_r02, 0.2199999988079071f, _v100037);
        const float _v100039 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100040 = __fmaf_rn(F2_r11, 0.0f, _v100039);
        const float s4_y = __fmaf_rn(F2_r12, 0.2199999988079071f, _v100040);
        const float _v100042 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100043 = __fmaf_rn(0.0f, 0.0f, _v100042);
        const float s4_z = __fmaf_rn(F2_r22, 0.2199999988079071f, _v100043);
        out[4] = make_float4(s4_x, s4_y, s4_z, 0.03999999910593033f);
        const float _v100045 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100046 = __fmaf_rn(F2_r01, 0.0f, _v100045);
        const float s5_x = __fmaf_rn(F2_r02, 0.25999999046325684f, _v100046);
        const float _v100048 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100049 = __fmaf_rn(F2_r11, 0.0f, _v100048);
        const float s5_y = __fmaf_rn(F2_r12, 0.25999999046325684f, _v100049);
        const float _v100051 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100052 = __fmaf_rn(0.0f, 0.0f, _v100051);
        const float s5_z = __fmaf_rn(F2_r22, 0.25999999046325684f, _v100052);
        out[5] = make_float4(s5_x, s5_y, s5_z, 0.03999999910593033f);
        const float _v100054 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100055 = __fmaf_rn(F2_r01, 0.0f, _v100054);
        const float s6_x = __fmaf_rn(F2_r02, 0.30000001192092896f, _v100055);
        const float _v100057 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100058 = __fmaf_rn(F2_r11, 0.0f, _v100057);
        const float s6_y = __fmaf_rn(F2_r12, 0.30000001192092896f, _v100058);
        const float _v100060 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100061 = __fmaf_rn(0.0f, 0.0f, _v100060);
        const float s6_z = __fmaf_rn(F2_r22, 0.30000001192092896f, _v100061);
        out[6] = make_float4(s6_x, s6_y, s6_z, 0.03999999910593033f);
        const float _v100063 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100064 = __fmaf_rn(F2_r01, 0.0f, _v100063);
        const float s7_x = __fmaf_rn(F2_r02, 0.3400000035762787f, _v100064);
        const float _v100066 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100067 = __fmaf_rn(F2_r11, 0.0f, _v100066);
        const float s7_y = __fmaf_rn(F2_r12, 0.3400000035762787f, _v100067);
        const float _v100069 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100070 = __fmaf_rn(0.0f, 0.0f, _v100069);
        const float s7_z = __fmaf_rn(F2_r22, 0.3400000035762787f, _v100070);
        out[7] = make_float4(s7_x, s7_y, s7_z, 0.03999999910593033f);
        const float _v100072 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
        const float _v100073 = __fmaf_rn(F2_r01, 0.0f, _v100072);
        const float s8_x = __fmaf_rn(F2_r02, 0.3799999952316284f, _v100073);
        const float _v100075 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
        const float _v100076 = __fmaf_rn(F2_r11, 0.0f, _v100075);
        const float s8_y = __fmaf_rn(F2_r12, 0.3799999952316284f, _v100076);
        const float _v100078 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
        const float _v100079 = __fmaf_rn(0.0f, 0.0f, _v100078);
        const float s8_z = __fmaf_rn(F2_r22, 0.3799999952316284f, _v100079);
        out[8] = make_float4(s8_x, s8_y, s8_z, 0.03999999910593033f);
    }
    // fine spheres [2, 3, 4, 5, 6] (upper_arm_link)
    static __device__ __noinline__ void fine_14(const float F1_r00, const float F1_r01, const float F1_r02, const float F1_r10, const float F1_r11, const float F1_r12, const float F1_r20, const float F1_r22, const float F1_t0, const float F1_t1, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v100001 = __fmaf_rn(F1_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(F1_r02, 0.10499999672174454f, _v100001);
        const float _v100003 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v100004 = __fmaf_rn(F1_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(F1_r12, 0.10499999672174454f, _v100004);
        const float _v100006 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v100007 = __fmaf_rn(0.0f, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(F1_r22, 0.10499999672174454f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.07999999821186066f);
        const float _v100009 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v100010 = __fmaf_rn(F1_r01, 0.0f, _v100009);
        const float s1_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v100010);
        const float _v100012 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v100013 = __fmaf_rn(F1_r11, 0.0f, _v100012);
        const float s1_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v100013);
        const float _v100015 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v100016 = __fmaf_rn(0.0f, 0.0f, _v100015);
        const float s1_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v100016);
        out[1] = make_float4(s1_x, s1_y, s1_z, 0.07999999821186066f);
        const float _v100018 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v100019 = __fmaf_rn(F1_r01, 0.0f, _v100018);
        const float s2_x = __fmaf_rn(F1_r02, 0.3149999976158142f, _v100019);
        const float _v100021 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v100022 = __fmaf_rn(F1_r11, 0.0f, _v100021);
        const float s2_y = __fmaf_rn(F1_r12, 0.3149999976158142f, _v100022);
        const float _v100024 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v100025 = __fmaf_rn(0.0f, 0.0f, _v100024);
        const float s2_z = __fmaf_rn(F1_r22, 0.3149999976158142f, _v100025);
        out[2] = make_float4(s2_x, s2_y, s2_z, 0.07999999821186066f);
        const float _v100027 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v100028 = __fmaf_rn(F1_r01, 0.0f, _v100027);
        const float s3_x = __fmaf_rn(F1_r02, 0.41999998688697815f, _v100028);
        const float _v100030 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v100031 = __fmaf_rn(F1_r11, 0.0f, _v100030);
        const float s3_y = __fmaf_rn(F1_r12, 0.41999998688697815f, _v100031);
        const float _v100033 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v100034 = __fmaf_rn(0.0f, 0.0f, _v100033);
        const float s3_z = __fmaf_rn(F1_r22, 0.41999998688697815f, _v100034);
        out[3] = make_float4(s3_x, s3_y, s3_z, 0.07999999821186066f);
        const float _v100036 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
        const float _v100037 = __fmaf_rn(F1_r01, 0.0f, _v100036);
        const float s4_x = __fmaf_rn(F1_r02, 0.0f, _v100037);
        const float _v100039 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
        const float _v100040 = __fmaf_rn(F1_r11, 0.0f, _v100039);
        const float s4_y = __fmaf_rn(F1_r12, 0.0f, _v100040);
        const float _v100042 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
        const float _v100043 = __fmaf_rn(0.0f, 0.0f, _v100042);
        const float s4_z = __fmaf_rn(F1_r22, 0.0f, _v100043);
        out[4] = make_float4(s4_x, s4_y, s4_z, 0.07999999821186066f);
    }
    // fine spheres [1] (shoulder_link)
    static __device__ __noinline__ void fine_15(const float F0_r00, const float F0_r01, const float F0_r10, const float F0_r11, float4 *out)
    {
        const float _v100000 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
        const float _v100001 = __fmaf_rn(F0_r01, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(0.0f, 0.0f, _v100001);
        const float _v100003 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
        const float _v100004 = __fmaf_rn(F0_r11, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(0.0f, 0.0f, _v100004);
        const float _v100006 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
        const float _v100007 = __fmaf_rn(0.0f, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(1.0f, 0.0f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.07999999821186066f);
    }
    // fine spheres [0] (base_link)
    static __device__ __noinline__ void fine_16(float4 *out)
    {
        const float _v100000 = __fmaf_rn(1.0f, 0.0f, 0.0f);
        const float _v100001 = __fmaf_rn(0.0f, 0.0f, _v100000);
        const float s0_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v100001);
        const float _v100003 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v100004 = __fmaf_rn(1.0f, 0.0f, _v100003);
        const float s0_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v100004);
        const float _v100006 = __fmaf_rn(0.0f, 0.0f, 0.0f);
        const float _v100007 = __fmaf_rn(0.0f, 0.0f, _v100006);
        const float s0_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v100007);
        out[0] = make_float4(s0_x, s0_y, s0_z, 0.07999999821186066f);
    }

    // Robot::fkcc for the lanes of ctx.alive.  Clears the lanes of every segment found in collision.
    template <typename Ctx>
    static __device__ __forceinline__ void fkcc(const float *q, Ctx &ctx)
    {
        float F0_s, F0_c; vg_sincos_ref(q[0], &F0_s, &F0_c);
        const float _v0 = __fmul_rn(0.0007963267271406949f, F0_c);
        const float F0_r00 = __fmaf_rn(-0.9999997019767761f, F0_s, _v0);
        const float _v2 = __fmul_rn(-0.0007963267271406949f, F0_s);
        const float F0_r01 = __fmaf_rn(-0.9999997019767761f, F0_c, _v2);
        const float _v4 = __fmul_rn(0.9999997019767761f, F0_c);
        const float F0_r10 = __fmaf_rn(0.0007963267271406949f, F0_s, _v4);
        const float _v6 = __fmul_rn(-0.9999997019767761f, F0_s);
        const float F0_r11 = __fmaf_rn(0.0007963267271406949f, F0_c, _v6);
        const float _v8 = __fmul_rn(0.1358499974012375f, F0_r01);
        const float _v9 = __fmul_rn(0.1358499974012375f, F0_r11);
        const float _v10 = __fmul_rn(1.7948965647107684e-09f, F0_r00);
        const float _v11 = __fmul_rn(1.7948965647107684e-09f, F0_r10);
        float F1_s, F1_c; vg_sincos_ref(q[1], &F1_s, &F1_c);
        const float _v12 = __fmul_rn(_v10, F1_c);
        const float F1_r00 = __fmaf_rn((-F0_r00), F1_s, _v12);
        const float F1_r01 = F0_r01;
        const float _v14 = __fmul_rn(_v10, F1_s);
        const float F1_r02 = __fmaf_rn(F0_r00, F1_c, _v14);
        const float _v16 = __fmul_rn(_v11, F1_c);
        const float F1_r10 = __fmaf_rn((-F0_r10), F1_s, _v16);
        const float F1_r11 = F0_r11;
        const float _v18 = __fmul_rn(_v11, F1_s);
        const float F1_r12 = __fmaf_rn(F0_r10, F1_c, _v18);
        const float F1_r20 = __fmaf_rn(-1.7948965647107684e-09f, F1_s, (-F1_c));
        const float F1_r22 = __fmaf_rn(1.7948965647107684e-09f, F1_c, (-F1_s));
        const float F1_t0 = _v8;
        const float F1_t1 = _v9;
        const float _v22 = __fmaf_rn(-0.11969999969005585f, F1_r01, F1_t0);
        const float _v23 = __fmaf_rn(0.42500001192092896f, F1_r02, _v22);
        const float _v24 = __fmaf_rn(-0.11969999969005585f, F1_r11, F1_t1);
        const float _v25 = __fmaf_rn(0.42500001192092896f, F1_r12, _v24);
        const float _v26 = __fmaf_rn(0.42500001192092896f, F1_r22, 1.0035589933395386f);
        float F2_s, F2_c; vg_sincos_ref(q[2], &F2_s, &F2_c);
        const float _v27 = __fmul_rn(F1_r00, F2_c);
        const float F2_r00 = __fmaf_rn((-F1_r02), F2_s, _v27);
        const float F2_r01 = F1_r01;
        const float _v29 = __fmul_rn(F1_r00, F2_s);
        const float F2_r02 = __fmaf_rn(F1_r02, F2_c, _v29);
        const float _v31 = __fmul_rn(F1_r10, F2_c);
        const float F2_r10 = __fmaf_rn((-F1_r12), F2_s, _v31);
        const float F2_r11 = F1_r11;
        const float _v33 = __fmul_rn(F1_r10, F2_s);
        const float F2_r12 = __fmaf_rn(F1_r12, F2_c, _v33);
        const float _v35 = __fmul_rn(F1_r20, F2_c);
        const float F2_r20 = __fmaf_rn((-F1_r22), F2_s, _v35);
        const float _v37 = __fmul_rn(F1_r20, F2_s);
        const float F2_r22 = __fmaf_rn(F1_r22, F2_c, _v37);
        const float F2_t0 = _v23;
        const float F2_t1 = _v25;
        const float F2_t2 = _v26;
        const float _v39 = __fmaf_rn(0.3922500014305115f, F2_r02, F2_t0);
        const float _v40 = __fmaf_rn(0.3922500014305115f, F2_r12, F2_t1);
        const float _v41 = __fmaf_rn(0.3922500014305115f, F2_r22, F2_t2);
        const float _v42 = __fmaf_rn(1.7948965647107684e-09f, F2_r00, (-F2_r02));
        const float _v43 = __fmaf_rn(1.7948965647107684e-09f, F2_r02, F2_r00);
        const float _v44 = __fmaf_rn(1.7948965647107684e-09f, F2_r10, (-F2_r12));
        const float _v45 = __fmaf_rn(1.7948965647107684e-09f, F2_r12, F2_r10);
        const float _v46 = __fmaf_rn(1.7948965647107684e-09f, F2_r20, (-F2_r22));
        const float _v47 = __fmaf_rn(1.7948965647107684e-09f, F2_r22, F2_r20);
        float F3_s, F3_c; vg_sincos_ref(q[3], &F3_s, &F3_c);
        const float _v48 = __fmul_rn(_v42, F3_c);
        const float F3_r00 = __fmaf_rn((-_v43), F3_s, _v48);
        const float F3_r01 = F2_r01;
        const float _v50 = __fmul_rn(_v42, F3_s);
        const float F3_r02 = __fmaf_rn(_v43, F3_c, _v50);
        const float _v52 = __fmul_rn(_v44, F3_c);
        const float F3_r10 = __fmaf_rn((-_v45), F3_s, _v52);
        const float F3_r11 = F2_r11;
        const float _v54 = __fmul_rn(_v44, F3_s);
        const float F3_r12 = __fmaf_rn(_v45, F3_c, _v54);
        const float _v56 = __fmul_rn(_v46, F3_c);
        const float F3_r20 = __fmaf_rn((-_v47), F3_s, _v56);
        const float _v58 = __fmul_rn(_v46, F3_s);
        const float F3_r22 = __fmaf_rn(_v47, F3_c, _v58);
        const float F3_t0 = _v39;
        const float F3_t1 = _v40;
        const float F3_t2 = _v41;
        const float _v60 = __fmaf_rn(0.09300000220537186f, F3_r01, F3_t0);
        const float _v61 = __fmaf_rn(0.09300000220537186f, F3_r11, F3_t1);
        float F4_s, F4_c; vg_sincos_ref(q[4], &F4_s, &F4_c);
        const float _v62 = __fmul_rn(F3_r00, F4_c);
        const float F4_r00 = __fmaf_rn(F3_r01, F4_s, _v62);
        const float _v64 = __fmul_rn((-F3_r00), F4_s);
        const float F4_r01 = __fmaf_rn(F3_r01, F4_c, _v64);
        const float F4_r02 = F3_r02;
        const float _v66 = __fmul_rn(F3_r10, F4_c);
        const float F4_r10 = __fmaf_rn(F3_r11, F4_s, _v66);
        const float _v68 = __fmul_rn((-F3_r10), F4_s);
        const float F4_r11 = __fmaf_rn(F3_r11, F4_c, _v68);
        const float F4_r12 = F3_r12;
        const float F4_r20 = __fmul_rn(F3_r20, F4_c);
        const float F4_r21 = __fmul_rn((-F3_r20), F4_s);
        const float F4_r22 = F3_r22;
        const float F4_t0 = _v60;
        const float F4_t1 = _v61;
        const float F4_t2 = F3_t2;
        const float _v72 = __fmaf_rn(0.09465000033378601f, F4_r02, F4_t0);
        const float _v73 = __fmaf_rn(0.09465000033378601f, F4_r12, F4_t1);
        const float _v74 = __fmaf_rn(0.09465000033378601f, F4_r22, F4_t2);
        float F5_s, F5_c; vg_sincos_ref(q[5], &F5_s, &F5_c);
        const float _v75 = __fmul_rn(F4_r00, F5_c);
        const float F5_r00 = __fmaf_rn((-F4_r02), F5_s, _v75);
        const float F5_r01 = F4_r01;
        const float _v77 = __fmul_rn(F4_r00, F5_s);
        const float F5_r02 = __fmaf_rn(F4_r02, F5_c, _v77);
        const float _v79 = __fmul_rn(F4_r10, F5_c);
        const float F5_r10 = __fmaf_rn((-F4_r12), F5_s, _v79);
        const float F5_r11 = F4_r11;
        const float _v81 = __fmul_rn(F4_r10, F5_s);
        const float F5_r12 = __fmaf_rn(F4_r12, F5_c, _v81);
        const float _v83 = __fmul_rn(F4_r20, F5_c);
        const float F5_r20 = __fmaf_rn((-F4_r22), F5_s, _v83);
        const float F5_r21 = F4_r21;
        const float _v85 = __fmul_rn(F4_r20, F5_s);
        const float F5_r22 = __fmaf_rn(F4_r22, F5_c, _v85);
        const float F5_t0 = _v72;
        const float F5_t1 = _v73;
        const float F5_t2 = _v74;
        float4 sa[9], sb[9];  // fine sphere scratch, reused by every check
        // environment: robotiq_85_right_finger_link
        {
            const float _v87 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
            const float _v88 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v87);
            const float c40_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v88);
            const float _v90 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
            const float _v91 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v90);
            const float c40_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v91);
            const float _v93 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
            const float _v94 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v93);
            const float c40_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v94);
            const unsigned need = ctx.env_hit(c40_x, c40_y, c40_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_0(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<3>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_right_knuckle_link
        {
            const float _v96 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
            const float _v97 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v96);
            const float c41_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v97);
            const float _v99 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
            const float _v100 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v99);
            const float c41_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v100);
            const float _v102 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
            const float _v103 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v102);
            const float c41_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v103);
            const unsigned need = ctx.env_hit(c41_x, c41_y, c41_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_1(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_right_finger_tip_link
        {
            const float _v105 = __fmaf_rn(F5_r00, -0.0469076968729496f, F5_t0);
            const float _v106 = __fmaf_rn(F5_r01, 0.2449275404214859f, _v105);
            const float c42_x = __fmaf_rn(F5_r02, 0.0006016629631631076f, _v106);
            const float _v108 = __fmaf_rn(F5_r10, -0.0469076968729496f, F5_t1);
            const float _v109 = __fmaf_rn(F5_r11, 0.2449275404214859f, _v108);
            const float c42_y = __fmaf_rn(F5_r12, 0.0006016629631631076f, _v109);
            const float _v111 = __fmaf_rn(F5_r20, -0.0469076968729496f, F5_t2);
            const float _v112 = __fmaf_rn(F5_r21, 0.2449275404214859f, _v111);
            const float c42_z = __fmaf_rn(F5_r22, 0.0006016629631631076f, _v112);
            const unsigned need = ctx.env_hit(c42_x, c42_y, c42_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_2(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<2>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_right_inner_knuckle_link
        {
            const float _v114 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
            const float _v115 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v114);
            const float c43_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v115);
            const float _v117 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
            const float _v118 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v117);
            const float c43_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v118);
            const float _v120 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
            const float _v121 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v120);
            const float c43_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v121);
            const unsigned need = ctx.env_hit(c43_x, c43_y, c43_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_3(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_left_finger_link
        {
            const float _v123 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
            const float _v124 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v123);
            const float c44_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v124);
            const float _v126 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
            const float _v127 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v126);
            const float c44_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v127);
            const float _v129 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
            const float _v130 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v129);
            const float c44_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v130);
            const unsigned need = ctx.env_hit(c44_x, c44_y, c44_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<3>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_left_knuckle_link
        {
            const float _v132 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
            const float _v133 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v132);
            const float c45_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v133);
            const float _v135 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
            const float _v136 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v135);
            const float c45_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v136);
            const float _v138 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
            const float _v139 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v138);
            const float c45_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v139);
            const unsigned need = ctx.env_hit(c45_x, c45_y, c45_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_5(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_left_finger_tip_link
        {
            const float _v141 = __fmaf_rn(F5_r00, 0.047183919697999954f, F5_t0);
            const float _v142 = __fmaf_rn(F5_r01, 0.24464209377765656f, _v141);
            const float c46_x = __fmaf_rn(F5_r02, 0.0006013759993948042f, _v142);
            const float _v144 = __fmaf_rn(F5_r10, 0.047183919697999954f, F5_t1);
            const float _v145 = __fmaf_rn(F5_r11, 0.24464209377765656f, _v144);
            const float c46_y = __fmaf_rn(F5_r12, 0.0006013759993948042f, _v145);
            const float _v147 = __fmaf_rn(F5_r20, 0.047183919697999954f, F5_t2);
            const float _v148 = __fmaf_rn(F5_r21, 0.24464209377765656f, _v147);
            const float c46_z = __fmaf_rn(F5_r22, 0.0006013759993948042f, _v148);
            const unsigned need = ctx.env_hit(c46_x, c46_y, c46_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_6(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<2>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_left_inner_knuckle_link
        {
            const float _v150 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
            const float _v151 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v150);
            const float c47_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v151);
            const float _v153 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
            const float _v154 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v153);
            const float c47_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v154);
            const float _v156 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
            const float _v157 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v156);
            const float c47_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v157);
            const unsigned need = ctx.env_hit(c47_x, c47_y, c47_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_7(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: robotiq_85_base_link
        {
            const float _v159 = __fmaf_rn(F5_r00, -3.185292371199466e-05f, F5_t0);
            const float _v160 = __fmaf_rn(F5_r01, 0.1572999805212021f, _v159);
            const float c48_x = __fmaf_rn(F5_r02, 0.0005318530602380633f, _v160);
            const float _v162 = __fmaf_rn(F5_r10, -3.185292371199466e-05f, F5_t1);
            const float _v163 = __fmaf_rn(F5_r11, 0.1572999805212021f, _v162);
            const float c48_y = __fmaf_rn(F5_r12, 0.0005318530602380633f, _v163);
            const float _v165 = __fmaf_rn(F5_r20, -3.185292371199466e-05f, F5_t2);
            const float _v166 = __fmaf_rn(F5_r21, 0.1572999805212021f, _v165);
            const float c48_z = __fmaf_rn(F5_r22, 0.0005318530602380633f, _v166);
            const unsigned need = ctx.env_hit(c48_x, c48_y, c48_z, 0.05999999865889549f, ctx.alive);
            if (need)
            {
                fine_8(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<2>(ctx, sa, need)) return;
            }
        }
        // environment: fts_robotside
        {
            const float _v168 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
            const float _v169 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v168);
            const float c49_x = __fmaf_rn(F5_r02, 0.0f, _v169);
            const float _v171 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
            const float _v172 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v171);
            const float c49_y = __fmaf_rn(F5_r12, 0.0f, _v172);
            const float _v174 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
            const float _v175 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v174);
            const float c49_z = __fmaf_rn(F5_r22, 0.0f, _v175);
            const unsigned need = ctx.env_hit(c49_x, c49_y, c49_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_9(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: wrist_3_link
        {
            const float _v177 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
            const float _v178 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v177);
            const float c50_x = __fmaf_rn(F5_r02, 0.0f, _v178);
            const float _v180 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
            const float _v181 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v180);
            const float c50_y = __fmaf_rn(F5_r12, 0.0f, _v181);
            const float _v183 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
            const float _v184 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v183);
            const float c50_z = __fmaf_rn(F5_r22, 0.0f, _v184);
            const unsigned need = ctx.env_hit(c50_x, c50_y, c50_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_10(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: wrist_2_link
        {
            const float _v186 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v187 = __fmaf_rn(F4_r01, 0.0f, _v186);
            const float c51_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v187);
            const float _v189 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v190 = __fmaf_rn(F4_r11, 0.0f, _v189);
            const float c51_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v190);
            const float _v192 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v193 = __fmaf_rn(F4_r21, 0.0f, _v192);
            const float c51_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v193);
            const unsigned need = ctx.env_hit(c51_x, c51_y, c51_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_11(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sa);
                if (vg::env_fine<3>(ctx, sa, need)) return;
            }
        }
        // environment: wrist_1_link
        {
            const float _v195 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
            const float _v196 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v195);
            const float c52_x = __fmaf_rn(F3_r02, 0.0f, _v196);
            const float _v198 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
            const float _v199 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v198);
            const float c52_y = __fmaf_rn(F3_r12, 0.0f, _v199);
            const float _v201 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
            const float _v202 = __fmaf_rn(0.0f, 0.09000000357627869f, _v201);
            const float c52_z = __fmaf_rn(F3_r22, 0.0f, _v202);
            const unsigned need = ctx.env_hit(c52_x, c52_y, c52_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_12(F3_r00, F3_r01, F3_r02, F3_r10, F3_r11, F3_r12, F3_r20, F3_r22, F3_t0, F3_t1, F3_t2, sa);
                if (vg::env_fine<3>(ctx, sa, need)) return;
            }
        }
        // environment: forearm_link
        {
            const float _v204 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v205 = __fmaf_rn(F2_r01, 0.0f, _v204);
            const float c53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v205);
            const float _v207 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v208 = __fmaf_rn(F2_r11, 0.0f, _v207);
            const float c53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v208);
            const float _v210 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v211 = __fmaf_rn(0.0f, 0.0f, _v210);
            const float c53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v211);
            const unsigned need = ctx.env_hit(c53_x, c53_y, c53_z, 0.25f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                if (vg::env_fine<9>(ctx, sa, need)) return;
            }
        }
        // environment: upper_arm_link
        {
            const float _v213 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v214 = __fmaf_rn(F1_r01, 0.0f, _v213);
            const float c54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v214);
            const float _v216 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v217 = __fmaf_rn(F1_r11, 0.0f, _v216);
            const float c54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v217);
            const float _v219 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v220 = __fmaf_rn(0.0f, 0.0f, _v219);
            const float c54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v220);
            const unsigned need = ctx.env_hit(c54_x, c54_y, c54_z, 0.28999999165534973f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                if (vg::env_fine<5>(ctx, sa, need)) return;
            }
        }
        // environment: shoulder_link
        {
            const float _v222 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v223 = __fmaf_rn(F0_r01, 0.0f, _v222);
            const float c55_x = __fmaf_rn(0.0f, 0.0f, _v223);
            const float _v225 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v226 = __fmaf_rn(F0_r11, 0.0f, _v225);
            const float c55_y = __fmaf_rn(0.0f, 0.0f, _v226);
            const float _v228 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v229 = __fmaf_rn(0.0f, 0.0f, _v228);
            const float c55_z = __fmaf_rn(1.0f, 0.0f, _v229);
            const unsigned need = ctx.env_hit(c55_x, c55_y, c55_z, 0.07999999821186066f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // environment: base_link
        {
            const float _v231 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v232 = __fmaf_rn(0.0f, 0.0f, _v231);
            const float c56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v232);
            const float _v234 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v235 = __fmaf_rn(1.0f, 0.0f, _v234);
            const float c56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v235);
            const float _v237 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v238 = __fmaf_rn(0.0f, 0.0f, _v237);
            const float c56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v238);
            const unsigned need = ctx.env_hit(c56_x, c56_y, c56_z, 0.07999999821186066f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                if (vg::env_fine<1>(ctx, sa, need)) return;
            }
        }
        // self: base_link vs. upper_arm_link
        {
            const float _v240 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v241 = __fmaf_rn(0.0f, 0.0f, _v240);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v241);
            const float _v243 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v244 = __fmaf_rn(1.0f, 0.0f, _v243);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v244);
            const float _v246 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v247 = __fmaf_rn(0.0f, 0.0f, _v246);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v247);
            const float _v249 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v250 = __fmaf_rn(F1_r01, 0.0f, _v249);
            const float cb54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v250);
            const float _v252 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v253 = __fmaf_rn(F1_r11, 0.0f, _v252);
            const float cb54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v253);
            const float _v255 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v256 = __fmaf_rn(0.0f, 0.0f, _v255);
            const float cb54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v256);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb54_x, cb54_y, cb54_z, 0.28999999165534973f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sb);
                if (vg::self_cross<1, 5>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. forearm_link
        {
            const float _v258 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v259 = __fmaf_rn(0.0f, 0.0f, _v258);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v259);
            const float _v261 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v262 = __fmaf_rn(1.0f, 0.0f, _v261);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v262);
            const float _v264 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v265 = __fmaf_rn(0.0f, 0.0f, _v264);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v265);
            const float _v267 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v268 = __fmaf_rn(F2_r01, 0.0f, _v267);
            const float cb53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v268);
            const float _v270 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v271 = __fmaf_rn(F2_r11, 0.0f, _v270);
            const float cb53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v271);
            const float _v273 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v274 = __fmaf_rn(0.0f, 0.0f, _v273);
            const float cb53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v274);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb53_x, cb53_y, cb53_z, 0.25f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sb);
                if (vg::self_cross<1, 9>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. wrist_1_link
        {
            const float _v276 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v277 = __fmaf_rn(0.0f, 0.0f, _v276);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v277);
            const float _v279 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v280 = __fmaf_rn(1.0f, 0.0f, _v279);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v280);
            const float _v282 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v283 = __fmaf_rn(0.0f, 0.0f, _v282);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v283);
            const float _v285 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
            const float _v286 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v285);
            const float cb52_x = __fmaf_rn(F3_r02, 0.0f, _v286);
            const float _v288 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
            const float _v289 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v288);
            const float cb52_y = __fmaf_rn(F3_r12, 0.0f, _v289);
            const float _v291 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
            const float _v292 = __fmaf_rn(0.0f, 0.09000000357627869f, _v291);
            const float cb52_z = __fmaf_rn(F3_r22, 0.0f, _v292);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb52_x, cb52_y, cb52_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_12(F3_r00, F3_r01, F3_r02, F3_r10, F3_r11, F3_r12, F3_r20, F3_r22, F3_t0, F3_t1, F3_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. wrist_2_link
        {
            const float _v294 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v295 = __fmaf_rn(0.0f, 0.0f, _v294);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v295);
            const float _v297 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v298 = __fmaf_rn(1.0f, 0.0f, _v297);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v298);
            const float _v300 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v301 = __fmaf_rn(0.0f, 0.0f, _v300);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v301);
            const float _v303 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v304 = __fmaf_rn(F4_r01, 0.0f, _v303);
            const float cb51_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v304);
            const float _v306 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v307 = __fmaf_rn(F4_r11, 0.0f, _v306);
            const float cb51_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v307);
            const float _v309 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v310 = __fmaf_rn(F4_r21, 0.0f, _v309);
            const float cb51_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v310);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb51_x, cb51_y, cb51_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_11(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. wrist_3_link
        {
            const float _v312 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v313 = __fmaf_rn(0.0f, 0.0f, _v312);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v313);
            const float _v315 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v316 = __fmaf_rn(1.0f, 0.0f, _v315);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v316);
            const float _v318 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v319 = __fmaf_rn(0.0f, 0.0f, _v318);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v319);
            const float _v321 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
            const float _v322 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v321);
            const float cb50_x = __fmaf_rn(F5_r02, 0.0f, _v322);
            const float _v324 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
            const float _v325 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v324);
            const float cb50_y = __fmaf_rn(F5_r12, 0.0f, _v325);
            const float _v327 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
            const float _v328 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v327);
            const float cb50_z = __fmaf_rn(F5_r22, 0.0f, _v328);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb50_x, cb50_y, cb50_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_10(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. fts_robotside
        {
            const float _v330 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v331 = __fmaf_rn(0.0f, 0.0f, _v330);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v331);
            const float _v333 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v334 = __fmaf_rn(1.0f, 0.0f, _v333);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v334);
            const float _v336 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v337 = __fmaf_rn(0.0f, 0.0f, _v336);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v337);
            const float _v339 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
            const float _v340 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v339);
            const float cb49_x = __fmaf_rn(F5_r02, 0.0f, _v340);
            const float _v342 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
            const float _v343 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v342);
            const float cb49_y = __fmaf_rn(F5_r12, 0.0f, _v343);
            const float _v345 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
            const float _v346 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v345);
            const float cb49_z = __fmaf_rn(F5_r22, 0.0f, _v346);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb49_x, cb49_y, cb49_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_9(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_base_link
        {
            const float _v348 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v349 = __fmaf_rn(0.0f, 0.0f, _v348);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v349);
            const float _v351 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v352 = __fmaf_rn(1.0f, 0.0f, _v351);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v352);
            const float _v354 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v355 = __fmaf_rn(0.0f, 0.0f, _v354);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v355);
            const float _v357 = __fmaf_rn(F5_r00, -3.185292371199466e-05f, F5_t0);
            const float _v358 = __fmaf_rn(F5_r01, 0.1572999805212021f, _v357);
            const float cb48_x = __fmaf_rn(F5_r02, 0.0005318530602380633f, _v358);
            const float _v360 = __fmaf_rn(F5_r10, -3.185292371199466e-05f, F5_t1);
            const float _v361 = __fmaf_rn(F5_r11, 0.1572999805212021f, _v360);
            const float cb48_y = __fmaf_rn(F5_r12, 0.0005318530602380633f, _v361);
            const float _v363 = __fmaf_rn(F5_r20, -3.185292371199466e-05f, F5_t2);
            const float _v364 = __fmaf_rn(F5_r21, 0.1572999805212021f, _v363);
            const float cb48_z = __fmaf_rn(F5_r22, 0.0005318530602380633f, _v364);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb48_x, cb48_y, cb48_z, 0.05999999865889549f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_8(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_left_inner_knuckle_link
        {
            const float _v366 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v367 = __fmaf_rn(0.0f, 0.0f, _v366);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v367);
            const float _v369 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v370 = __fmaf_rn(1.0f, 0.0f, _v369);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v370);
            const float _v372 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v373 = __fmaf_rn(0.0f, 0.0f, _v372);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v373);
            const float _v375 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
            const float _v376 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v375);
            const float cb47_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v376);
            const float _v378 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
            const float _v379 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v378);
            const float cb47_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v379);
            const float _v381 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
            const float _v382 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v381);
            const float cb47_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v382);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb47_x, cb47_y, cb47_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_7(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_left_finger_tip_link
        {
            const float _v384 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v385 = __fmaf_rn(0.0f, 0.0f, _v384);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v385);
            const float _v387 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v388 = __fmaf_rn(1.0f, 0.0f, _v387);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v388);
            const float _v390 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v391 = __fmaf_rn(0.0f, 0.0f, _v390);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v391);
            const float _v393 = __fmaf_rn(F5_r00, 0.047183919697999954f, F5_t0);
            const float _v394 = __fmaf_rn(F5_r01, 0.24464209377765656f, _v393);
            const float cb46_x = __fmaf_rn(F5_r02, 0.0006013759993948042f, _v394);
            const float _v396 = __fmaf_rn(F5_r10, 0.047183919697999954f, F5_t1);
            const float _v397 = __fmaf_rn(F5_r11, 0.24464209377765656f, _v396);
            const float cb46_y = __fmaf_rn(F5_r12, 0.0006013759993948042f, _v397);
            const float _v399 = __fmaf_rn(F5_r20, 0.047183919697999954f, F5_t2);
            const float _v400 = __fmaf_rn(F5_r21, 0.24464209377765656f, _v399);
            const float cb46_z = __fmaf_rn(F5_r22, 0.0006013759993948042f, _v400);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb46_x, cb46_y, cb46_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_6(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_left_knuckle_link
        {
            const float _v402 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v403 = __fmaf_rn(0.0f, 0.0f, _v402);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v403);
            const float _v405 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v406 = __fmaf_rn(1.0f, 0.0f, _v405);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v406);
            const float _v408 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v409 = __fmaf_rn(0.0f, 0.0f, _v408);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v409);
            const float _v411 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
            const float _v412 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v411);
            const float cb45_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v412);
            const float _v414 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
            const float _v415 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v414);
            const float cb45_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v415);
            const float _v417 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
            const float _v418 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v417);
            const float cb45_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v418);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb45_x, cb45_y, cb45_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_5(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_left_finger_link
        {
            const float _v420 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v421 = __fmaf_rn(0.0f, 0.0f, _v420);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v421);
            const float _v423 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v424 = __fmaf_rn(1.0f, 0.0f, _v423);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v424);
            const float _v426 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v427 = __fmaf_rn(0.0f, 0.0f, _v426);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v427);
            const float _v429 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
            const float _v430 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v429);
            const float cb44_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v430);
            const float _v432 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
            const float _v433 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v432);
            const float cb44_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v433);
            const float _v435 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
            const float _v436 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v435);
            const float cb44_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v436);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb44_x, cb44_y, cb44_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_right_inner_knuckle_link
        {
            const float _v438 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v439 = __fmaf_rn(0.0f, 0.0f, _v438);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v439);
            const float _v441 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v442 = __fmaf_rn(1.0f, 0.0f, _v441);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v442);
            const float _v444 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v445 = __fmaf_rn(0.0f, 0.0f, _v444);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v445);
            const float _v447 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
            const float _v448 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v447);
            const float cb43_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v448);
            const float _v450 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
            const float _v451 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v450);
            const float cb43_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v451);
            const float _v453 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
            const float _v454 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v453);
            const float cb43_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v454);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb43_x, cb43_y, cb43_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_3(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_right_finger_tip_link
        {
            const float _v456 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v457 = __fmaf_rn(0.0f, 0.0f, _v456);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v457);
            const float _v459 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v460 = __fmaf_rn(1.0f, 0.0f, _v459);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v460);
            const float _v462 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v463 = __fmaf_rn(0.0f, 0.0f, _v462);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v463);
            const float _v465 = __fmaf_rn(F5_r00, -0.0469076968729496f, F5_t0);
            const float _v466 = __fmaf_rn(F5_r01, 0.2449275404214859f, _v465);
            const float cb42_x = __fmaf_rn(F5_r02, 0.0006016629631631076f, _v466);
            const float _v468 = __fmaf_rn(F5_r10, -0.0469076968729496f, F5_t1);
            const float _v469 = __fmaf_rn(F5_r11, 0.2449275404214859f, _v468);
            const float cb42_y = __fmaf_rn(F5_r12, 0.0006016629631631076f, _v469);
            const float _v471 = __fmaf_rn(F5_r20, -0.0469076968729496f, F5_t2);
            const float _v472 = __fmaf_rn(F5_r21, 0.2449275404214859f, _v471);
            const float cb42_z = __fmaf_rn(F5_r22, 0.0006016629631631076f, _v472);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb42_x, cb42_y, cb42_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_2(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_right_knuckle_link
        {
            const float _v474 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v475 = __fmaf_rn(0.0f, 0.0f, _v474);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v475);
            const float _v477 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v478 = __fmaf_rn(1.0f, 0.0f, _v477);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v478);
            const float _v480 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v481 = __fmaf_rn(0.0f, 0.0f, _v480);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v481);
            const float _v483 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
            const float _v484 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v483);
            const float cb41_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v484);
            const float _v486 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
            const float _v487 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v486);
            const float cb41_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v487);
            const float _v489 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
            const float _v490 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v489);
            const float cb41_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v490);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb41_x, cb41_y, cb41_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_1(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: base_link vs. robotiq_85_right_finger_link
        {
            const float _v492 = __fmaf_rn(1.0f, 0.0f, 0.0f);
            const float _v493 = __fmaf_rn(0.0f, 0.0f, _v492);
            const float ca56_x = __fmaf_rn(0.0f, 0.9143999814987183f, _v493);
            const float _v495 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v496 = __fmaf_rn(1.0f, 0.0f, _v495);
            const float ca56_y = __fmaf_rn(0.0f, 0.9143999814987183f, _v496);
            const float _v498 = __fmaf_rn(0.0f, 0.0f, 0.0f);
            const float _v499 = __fmaf_rn(0.0f, 0.0f, _v498);
            const float ca56_z = __fmaf_rn(1.0f, 0.9143999814987183f, _v499);
            const float _v501 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
            const float _v502 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v501);
            const float cb40_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v502);
            const float _v504 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
            const float _v505 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v504);
            const float cb40_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v505);
            const float _v507 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
            const float _v508 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v507);
            const float cb40_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v508);
            const unsigned need = ctx.self_hit(ca56_x, ca56_y, ca56_z, 0.07999999821186066f, cb40_x, cb40_y, cb40_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_16(sa);
                fine_0(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. forearm_link
        {
            const float _v510 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v511 = __fmaf_rn(F0_r01, 0.0f, _v510);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v511);
            const float _v513 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v514 = __fmaf_rn(F0_r11, 0.0f, _v513);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v514);
            const float _v516 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v517 = __fmaf_rn(0.0f, 0.0f, _v516);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v517);
            const float _v519 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v520 = __fmaf_rn(F2_r01, 0.0f, _v519);
            const float cb53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v520);
            const float _v522 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v523 = __fmaf_rn(F2_r11, 0.0f, _v522);
            const float cb53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v523);
            const float _v525 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v526 = __fmaf_rn(0.0f, 0.0f, _v525);
            const float cb53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v526);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb53_x, cb53_y, cb53_z, 0.25f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sb);
                if (vg::self_cross<1, 9>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. wrist_1_link
        {
            const float _v528 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v529 = __fmaf_rn(F0_r01, 0.0f, _v528);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v529);
            const float _v531 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v532 = __fmaf_rn(F0_r11, 0.0f, _v531);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v532);
            const float _v534 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v535 = __fmaf_rn(0.0f, 0.0f, _v534);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v535);
            const float _v537 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
            const float _v538 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v537);
            const float cb52_x = __fmaf_rn(F3_r02, 0.0f, _v538);
            const float _v540 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
            const float _v541 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v540);
            const float cb52_y = __fmaf_rn(F3_r12, 0.0f, _v541);
            const float _v543 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
            const float _v544 = __fmaf_rn(0.0f, 0.09000000357627869f, _v543);
            const float cb52_z = __fmaf_rn(F3_r22, 0.0f, _v544);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb52_x, cb52_y, cb52_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_12(F3_r00, F3_r01, F3_r02, F3_r10, F3_r11, F3_r12, F3_r20, F3_r22, F3_t0, F3_t1, F3_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. wrist_2_link
        {
            const float _v546 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v547 = __fmaf_rn(F0_r01, 0.0f, _v546);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v547);
            const float _v549 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v550 = __fmaf_rn(F0_r11, 0.0f, _v549);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v550);
            const float _v552 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v553 = __fmaf_rn(0.0f, 0.0f, _v552);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v553);
            const float _v555 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v556 = __fmaf_rn(F4_r01, 0.0f, _v555);
            const float cb51_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v556);
            const float _v558 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v559 = __fmaf_rn(F4_r11, 0.0f, _v558);
            const float cb51_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v559);
            const float _v561 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v562 = __fmaf_rn(F4_r21, 0.0f, _v561);
            const float cb51_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v562);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb51_x, cb51_y, cb51_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_11(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. wrist_3_link
        {
            const float _v564 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v565 = __fmaf_rn(F0_r01, 0.0f, _v564);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v565);
            const float _v567 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v568 = __fmaf_rn(F0_r11, 0.0f, _v567);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v568);
            const float _v570 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v571 = __fmaf_rn(0.0f, 0.0f, _v570);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v571);
            const float _v573 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
            const float _v574 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v573);
            const float cb50_x = __fmaf_rn(F5_r02, 0.0f, _v574);
            const float _v576 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
            const float _v577 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v576);
            const float cb50_y = __fmaf_rn(F5_r12, 0.0f, _v577);
            const float _v579 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
            const float _v580 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v579);
            const float cb50_z = __fmaf_rn(F5_r22, 0.0f, _v580);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb50_x, cb50_y, cb50_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_10(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. fts_robotside
        {
            const float _v582 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v583 = __fmaf_rn(F0_r01, 0.0f, _v582);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v583);
            const float _v585 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v586 = __fmaf_rn(F0_r11, 0.0f, _v585);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v586);
            const float _v588 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v589 = __fmaf_rn(0.0f, 0.0f, _v588);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v589);
            const float _v591 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
            const float _v592 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v591);
            const float cb49_x = __fmaf_rn(F5_r02, 0.0f, _v592);
            const float _v594 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
            const float _v595 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v594);
            const float cb49_y = __fmaf_rn(F5_r12, 0.0f, _v595);
            const float _v597 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
            const float _v598 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v597);
            const float cb49_z = __fmaf_rn(F5_r22, 0.0f, _v598);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb49_x, cb49_y, cb49_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_9(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_base_link
        {
            const float _v600 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v601 = __fmaf_rn(F0_r01, 0.0f, _v600);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v601);
            const float _v603 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v604 = __fmaf_rn(F0_r11, 0.0f, _v603);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v604);
            const float _v606 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v607 = __fmaf_rn(0.0f, 0.0f, _v606);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v607);
            const float _v609 = __fmaf_rn(F5_r00, -3.185292371199466e-05f, F5_t0);
            const float _v610 = __fmaf_rn(F5_r01, 0.1572999805212021f, _v609);
            const float cb48_x = __fmaf_rn(F5_r02, 0.0005318530602380633f, _v610);
            const float _v612 = __fmaf_rn(F5_r10, -3.185292371199466e-05f, F5_t1);
            const float _v613 = __fmaf_rn(F5_r11, 0.1572999805212021f, _v612);
            const float cb48_y = __fmaf_rn(F5_r12, 0.0005318530602380633f, _v613);
            const float _v615 = __fmaf_rn(F5_r20, -3.185292371199466e-05f, F5_t2);
            const float _v616 = __fmaf_rn(F5_r21, 0.1572999805212021f, _v615);
            const float cb48_z = __fmaf_rn(F5_r22, 0.0005318530602380633f, _v616);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb48_x, cb48_y, cb48_z, 0.05999999865889549f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_8(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_left_inner_knuckle_link
        {
            const float _v618 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v619 = __fmaf_rn(F0_r01, 0.0f, _v618);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v619);
            const float _v621 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v622 = __fmaf_rn(F0_r11, 0.0f, _v621);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v622);
            const float _v624 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v625 = __fmaf_rn(0.0f, 0.0f, _v624);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v625);
            const float _v627 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
            const float _v628 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v627);
            const float cb47_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v628);
            const float _v630 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
            const float _v631 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v630);
            const float cb47_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v631);
            const float _v633 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
            const float _v634 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v633);
            const float cb47_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v634);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb47_x, cb47_y, cb47_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_7(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_left_finger_tip_link
        {
            const float _v636 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v637 = __fmaf_rn(F0_r01, 0.0f, _v636);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v637);
            const float _v639 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v640 = __fmaf_rn(F0_r11, 0.0f, _v639);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v640);
            const float _v642 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v643 = __fmaf_rn(0.0f, 0.0f, _v642);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v643);
            const float _v645 = __fmaf_rn(F5_r00, 0.047183919697999954f, F5_t0);
            const float _v646 = __fmaf_rn(F5_r01, 0.24464209377765656f, _v645);
            const float cb46_x = __fmaf_rn(F5_r02, 0.0006013759993948042f, _v646);
            const float _v648 = __fmaf_rn(F5_r10, 0.047183919697999954f, F5_t1);
            const float _v649 = __fmaf_rn(F5_r11, 0.24464209377765656f, _v648);
            const float cb46_y = __fmaf_rn(F5_r12, 0.0006013759993948042f, _v649);
            const float _v651 = __fmaf_rn(F5_r20, 0.047183919697999954f, F5_t2);
            const float _v652 = __fmaf_rn(F5_r21, 0.24464209377765656f, _v651);
            const float cb46_z = __fmaf_rn(F5_r22, 0.0006013759993948042f, _v652);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb46_x, cb46_y, cb46_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_6(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_left_knuckle_link
        {
            const float _v654 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v655 = __fmaf_rn(F0_r01, 0.0f, _v654);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v655);
            const float _v657 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v658 = __fmaf_rn(F0_r11, 0.0f, _v657);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v658);
            const float _v660 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v661 = __fmaf_rn(0.0f, 0.0f, _v660);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v661);
            const float _v663 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
            const float _v664 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v663);
            const float cb45_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v664);
            const float _v666 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
            const float _v667 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v666);
            const float cb45_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v667);
            const float _v669 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
            const float _v670 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v669);
            const float cb45_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v670);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb45_x, cb45_y, cb45_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_5(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_left_finger_link
        {
            const float _v672 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v673 = __fmaf_rn(F0_r01, 0.0f, _v672);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v673);
            const float _v675 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v676 = __fmaf_rn(F0_r11, 0.0f, _v675);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v676);
            const float _v678 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v679 = __fmaf_rn(0.0f, 0.0f, _v678);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v679);
            const float _v681 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
            const float _v682 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v681);
            const float cb44_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v682);
            const float _v684 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
            const float _v685 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v684);
            const float cb44_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v685);
            const float _v687 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
            const float _v688 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v687);
            const float cb44_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v688);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb44_x, cb44_y, cb44_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_right_inner_knuckle_link
        {
            const float _v690 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v691 = __fmaf_rn(F0_r01, 0.0f, _v690);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v691);
            const float _v693 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v694 = __fmaf_rn(F0_r11, 0.0f, _v693);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v694);
            const float _v696 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v697 = __fmaf_rn(0.0f, 0.0f, _v696);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v697);
            const float _v699 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
            const float _v700 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v699);
            const float cb43_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v700);
            const float _v702 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
            const float _v703 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v702);
            const float cb43_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v703);
            const float _v705 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
            const float _v706 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v705);
            const float cb43_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v706);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb43_x, cb43_y, cb43_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_3(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_right_finger_tip_link
        {
            const float _v708 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v709 = __fmaf_rn(F0_r01, 0.0f, _v708);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v709);
            const float _v711 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v712 = __fmaf_rn(F0_r11, 0.0f, _v711);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v712);
            const float _v714 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v715 = __fmaf_rn(0.0f, 0.0f, _v714);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v715);
            const float _v717 = __fmaf_rn(F5_r00, -0.0469076968729496f, F5_t0);
            const float _v718 = __fmaf_rn(F5_r01, 0.2449275404214859f, _v717);
            const float cb42_x = __fmaf_rn(F5_r02, 0.0006016629631631076f, _v718);
            const float _v720 = __fmaf_rn(F5_r10, -0.0469076968729496f, F5_t1);
            const float _v721 = __fmaf_rn(F5_r11, 0.2449275404214859f, _v720);
            const float cb42_y = __fmaf_rn(F5_r12, 0.0006016629631631076f, _v721);
            const float _v723 = __fmaf_rn(F5_r20, -0.0469076968729496f, F5_t2);
            const float _v724 = __fmaf_rn(F5_r21, 0.2449275404214859f, _v723);
            const float cb42_z = __fmaf_rn(F5_r22, 0.0006016629631631076f, _v724);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb42_x, cb42_y, cb42_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_2(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_right_knuckle_link
        {
            const float _v726 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v727 = __fmaf_rn(F0_r01, 0.0f, _v726);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v727);
            const float _v729 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v730 = __fmaf_rn(F0_r11, 0.0f, _v729);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v730);
            const float _v732 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v733 = __fmaf_rn(0.0f, 0.0f, _v732);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v733);
            const float _v735 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
            const float _v736 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v735);
            const float cb41_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v736);
            const float _v738 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
            const float _v739 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v738);
            const float cb41_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v739);
            const float _v741 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
            const float _v742 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v741);
            const float cb41_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v742);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb41_x, cb41_y, cb41_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_1(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: shoulder_link vs. robotiq_85_right_finger_link
        {
            const float _v744 = __fmaf_rn(F0_r00, 0.0f, 0.0f);
            const float _v745 = __fmaf_rn(F0_r01, 0.0f, _v744);
            const float ca55_x = __fmaf_rn(0.0f, 0.0f, _v745);
            const float _v747 = __fmaf_rn(F0_r10, 0.0f, 0.0f);
            const float _v748 = __fmaf_rn(F0_r11, 0.0f, _v747);
            const float ca55_y = __fmaf_rn(0.0f, 0.0f, _v748);
            const float _v750 = __fmaf_rn(0.0f, 0.0f, 1.0035589933395386f);
            const float _v751 = __fmaf_rn(0.0f, 0.0f, _v750);
            const float ca55_z = __fmaf_rn(1.0f, 0.0f, _v751);
            const float _v753 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
            const float _v754 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v753);
            const float cb40_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v754);
            const float _v756 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
            const float _v757 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v756);
            const float cb40_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v757);
            const float _v759 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
            const float _v760 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v759);
            const float cb40_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v760);
            const unsigned need = ctx.self_hit(ca55_x, ca55_y, ca55_z, 0.07999999821186066f, cb40_x, cb40_y, cb40_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_15(F0_r00, F0_r01, F0_r10, F0_r11, sa);
                fine_0(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<1, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. wrist_1_link
        {
            const float _v762 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v763 = __fmaf_rn(F1_r01, 0.0f, _v762);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v763);
            const float _v765 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v766 = __fmaf_rn(F1_r11, 0.0f, _v765);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v766);
            const float _v768 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v769 = __fmaf_rn(0.0f, 0.0f, _v768);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v769);
            const float _v771 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
            const float _v772 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v771);
            const float cb52_x = __fmaf_rn(F3_r02, 0.0f, _v772);
            const float _v774 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
            const float _v775 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v774);
            const float cb52_y = __fmaf_rn(F3_r12, 0.0f, _v775);
            const float _v777 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
            const float _v778 = __fmaf_rn(0.0f, 0.09000000357627869f, _v777);
            const float cb52_z = __fmaf_rn(F3_r22, 0.0f, _v778);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb52_x, cb52_y, cb52_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_12(F3_r00, F3_r01, F3_r02, F3_r10, F3_r11, F3_r12, F3_r20, F3_r22, F3_t0, F3_t1, F3_t2, sb);
                if (vg::self_cross<5, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. wrist_2_link
        {
            const float _v780 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v781 = __fmaf_rn(F1_r01, 0.0f, _v780);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v781);
            const float _v783 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v784 = __fmaf_rn(F1_r11, 0.0f, _v783);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v784);
            const float _v786 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v787 = __fmaf_rn(0.0f, 0.0f, _v786);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v787);
            const float _v789 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v790 = __fmaf_rn(F4_r01, 0.0f, _v789);
            const float cb51_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v790);
            const float _v792 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v793 = __fmaf_rn(F4_r11, 0.0f, _v792);
            const float cb51_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v793);
            const float _v795 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v796 = __fmaf_rn(F4_r21, 0.0f, _v795);
            const float cb51_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v796);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb51_x, cb51_y, cb51_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_11(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<5, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. wrist_3_link
        {
            const float _v798 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v799 = __fmaf_rn(F1_r01, 0.0f, _v798);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v799);
            const float _v801 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v802 = __fmaf_rn(F1_r11, 0.0f, _v801);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v802);
            const float _v804 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v805 = __fmaf_rn(0.0f, 0.0f, _v804);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v805);
            const float _v807 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
            const float _v808 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v807);
            const float cb50_x = __fmaf_rn(F5_r02, 0.0f, _v808);
            const float _v810 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
            const float _v811 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v810);
            const float cb50_y = __fmaf_rn(F5_r12, 0.0f, _v811);
            const float _v813 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
            const float _v814 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v813);
            const float cb50_z = __fmaf_rn(F5_r22, 0.0f, _v814);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb50_x, cb50_y, cb50_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_10(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. fts_robotside
        {
            const float _v816 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v817 = __fmaf_rn(F1_r01, 0.0f, _v816);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v817);
            const float _v819 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v820 = __fmaf_rn(F1_r11, 0.0f, _v819);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v820);
            const float _v822 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v823 = __fmaf_rn(0.0f, 0.0f, _v822);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v823);
            const float _v825 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
            const float _v826 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v825);
            const float cb49_x = __fmaf_rn(F5_r02, 0.0f, _v826);
            const float _v828 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
            const float _v829 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v828);
            const float cb49_y = __fmaf_rn(F5_r12, 0.0f, _v829);
            const float _v831 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
            const float _v832 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v831);
            const float cb49_z = __fmaf_rn(F5_r22, 0.0f, _v832);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb49_x, cb49_y, cb49_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_9(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_base_link
        {
            const float _v834 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v835 = __fmaf_rn(F1_r01, 0.0f, _v834);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v835);
            const float _v837 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v838 = __fmaf_rn(F1_r11, 0.0f, _v837);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v838);
            const float _v840 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v841 = __fmaf_rn(0.0f, 0.0f, _v840);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v841);
            const float _v843 = __fmaf_rn(F5_r00, -3.185292371199466e-05f, F5_t0);
            const float _v844 = __fmaf_rn(F5_r01, 0.1572999805212021f, _v843);
            const float cb48_x = __fmaf_rn(F5_r02, 0.0005318530602380633f, _v844);
            const float _v846 = __fmaf_rn(F5_r10, -3.185292371199466e-05f, F5_t1);
            const float _v847 = __fmaf_rn(F5_r11, 0.1572999805212021f, _v846);
            const float cb48_y = __fmaf_rn(F5_r12, 0.0005318530602380633f, _v847);
            const float _v849 = __fmaf_rn(F5_r20, -3.185292371199466e-05f, F5_t2);
            const float _v850 = __fmaf_rn(F5_r21, 0.1572999805212021f, _v849);
            const float cb48_z = __fmaf_rn(F5_r22, 0.0005318530602380633f, _v850);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb48_x, cb48_y, cb48_z, 0.05999999865889549f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_8(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_left_inner_knuckle_link
        {
            const float _v852 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v853 = __fmaf_rn(F1_r01, 0.0f, _v852);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v853);
            const float _v855 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v856 = __fmaf_rn(F1_r11, 0.0f, _v855);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v856);
            const float _v858 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v859 = __fmaf_rn(0.0f, 0.0f, _v858);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v859);
            const float _v861 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
            const float _v862 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v861);
            const float cb47_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v862);
            const float _v864 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
            const float _v865 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v864);
            const float cb47_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v865);
            const float _v867 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
            const float _v868 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v867);
            const float cb47_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v868);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb47_x, cb47_y, cb47_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_7(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_left_finger_tip_link
        {
            const float _v870 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v871 = __fmaf_rn(F1_r01, 0.0f, _v870);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v871);
            const float _v873 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v874 = __fmaf_rn(F1_r11, 0.0f, _v873);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v874);
            const float _v876 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v877 = __fmaf_rn(0.0f, 0.0f, _v876);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v877);
            const float _v879 = __fmaf_rn(F5_r00, 0.047183919697999954f, F5_t0);
            const float _v880 = __fmaf_rn(F5_r01, 0.24464209377765656f, _v879);
            const float cb46_x = __fmaf_rn(F5_r02, 0.0006013759993948042f, _v880);
            const float _v882 = __fmaf_rn(F5_r10, 0.047183919697999954f, F5_t1);
            const float _v883 = __fmaf_rn(F5_r11, 0.24464209377765656f, _v882);
            const float cb46_y = __fmaf_rn(F5_r12, 0.0006013759993948042f, _v883);
            const float _v885 = __fmaf_rn(F5_r20, 0.047183919697999954f, F5_t2);
            const float _v886 = __fmaf_rn(F5_r21, 0.24464209377765656f, _v885);
            const float cb46_z = __fmaf_rn(F5_r22, 0.0006013759993948042f, _v886);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb46_x, cb46_y, cb46_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_6(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_left_knuckle_link
        {
            const float _v888 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v889 = __fmaf_rn(F1_r01, 0.0f, _v888);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v889);
            const float _v891 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v892 = __fmaf_rn(F1_r11, 0.0f, _v891);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v892);
            const float _v894 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v895 = __fmaf_rn(0.0f, 0.0f, _v894);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v895);
            const float _v897 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
            const float _v898 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v897);
            const float cb45_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v898);
            const float _v900 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
            const float _v901 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v900);
            const float cb45_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v901);
            const float _v903 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
            const float _v904 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v903);
            const float cb45_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v904);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb45_x, cb45_y, cb45_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_5(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_left_finger_link
        {
            const float _v906 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v907 = __fmaf_rn(F1_r01, 0.0f, _v906);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v907);
            const float _v909 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v910 = __fmaf_rn(F1_r11, 0.0f, _v909);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v910);
            const float _v912 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v913 = __fmaf_rn(0.0f, 0.0f, _v912);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v913);
            const float _v915 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
            const float _v916 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v915);
            const float cb44_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v916);
            const float _v918 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
            const float _v919 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v918);
            const float cb44_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v919);
            const float _v921 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
            const float _v922 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v921);
            const float cb44_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v922);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb44_x, cb44_y, cb44_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_right_inner_knuckle_link
        {
            const float _v924 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v925 = __fmaf_rn(F1_r01, 0.0f, _v924);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v925);
            const float _v927 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v928 = __fmaf_rn(F1_r11, 0.0f, _v927);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v928);
            const float _v930 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v931 = __fmaf_rn(0.0f, 0.0f, _v930);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v931);
            const float _v933 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
            const float _v934 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v933);
            const float cb43_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v934);
            const float _v936 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
            const float _v937 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v936);
            const float cb43_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v937);
            const float _v939 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
            const float _v940 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v939);
            const float cb43_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v940);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb43_x, cb43_y, cb43_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_3(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_right_finger_tip_link
        {
            const float _v942 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v943 = __fmaf_rn(F1_r01, 0.0f, _v942);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v943);
            const float _v945 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v946 = __fmaf_rn(F1_r11, 0.0f, _v945);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v946);
            const float _v948 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v949 = __fmaf_rn(0.0f, 0.0f, _v948);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v949);
            const float _v951 = __fmaf_rn(F5_r00, -0.0469076968729496f, F5_t0);
            const float _v952 = __fmaf_rn(F5_r01, 0.2449275404214859f, _v951);
            const float cb42_x = __fmaf_rn(F5_r02, 0.0006016629631631076f, _v952);
            const float _v954 = __fmaf_rn(F5_r10, -0.0469076968729496f, F5_t1);
            const float _v955 = __fmaf_rn(F5_r11, 0.2449275404214859f, _v954);
            const float cb42_y = __fmaf_rn(F5_r12, 0.0006016629631631076f, _v955);
            const float _v957 = __fmaf_rn(F5_r20, -0.0469076968729496f, F5_t2);
            const float _v958 = __fmaf_rn(F5_r21, 0.2449275404214859f, _v957);
            const float cb42_z = __fmaf_rn(F5_r22, 0.0006016629631631076f, _v958);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb42_x, cb42_y, cb42_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_2(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_right_knuckle_link
        {
            const float _v960 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v961 = __fmaf_rn(F1_r01, 0.0f, _v960);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v961);
            const float _v963 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v964 = __fmaf_rn(F1_r11, 0.0f, _v963);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v964);
            const float _v966 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v967 = __fmaf_rn(0.0f, 0.0f, _v966);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v967);
            const float _v969 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
            const float _v970 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v969);
            const float cb41_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v970);
            const float _v972 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
            const float _v973 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v972);
            const float cb41_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v973);
            const float _v975 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
            const float _v976 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v975);
            const float cb41_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v976);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb41_x, cb41_y, cb41_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_1(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: upper_arm_link vs. robotiq_85_right_finger_link
        {
            const float _v978 = __fmaf_rn(F1_r00, 0.0f, F1_t0);
            const float _v979 = __fmaf_rn(F1_r01, 0.0f, _v978);
            const float ca54_x = __fmaf_rn(F1_r02, 0.20999999344348907f, _v979);
            const float _v981 = __fmaf_rn(F1_r10, 0.0f, F1_t1);
            const float _v982 = __fmaf_rn(F1_r11, 0.0f, _v981);
            const float ca54_y = __fmaf_rn(F1_r12, 0.20999999344348907f, _v982);
            const float _v984 = __fmaf_rn(F1_r20, 0.0f, 1.0035589933395386f);
            const float _v985 = __fmaf_rn(0.0f, 0.0f, _v984);
            const float ca54_z = __fmaf_rn(F1_r22, 0.20999999344348907f, _v985);
            const float _v987 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
            const float _v988 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v987);
            const float cb40_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v988);
            const float _v990 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
            const float _v991 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v990);
            const float cb40_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v991);
            const float _v993 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
            const float _v994 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v993);
            const float cb40_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v994);
            const unsigned need = ctx.self_hit(ca54_x, ca54_y, ca54_z, 0.28999999165534973f, cb40_x, cb40_y, cb40_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_14(F1_r00, F1_r01, F1_r02, F1_r10, F1_r11, F1_r12, F1_r20, F1_r22, F1_t0, F1_t1, sa);
                fine_0(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<5, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. wrist_2_link
        {
            const float _v996 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v997 = __fmaf_rn(F2_r01, 0.0f, _v996);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v997);
            const float _v999 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1000 = __fmaf_rn(F2_r11, 0.0f, _v999);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1000);
            const float _v1002 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1003 = __fmaf_rn(0.0f, 0.0f, _v1002);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1003);
            const float _v1005 = __fmaf_rn(F4_r00, 0.0f, F4_t0);
            const float _v1006 = __fmaf_rn(F4_r01, 0.0f, _v1005);
            const float cb51_x = __fmaf_rn(F4_r02, 0.09000000357627869f, _v1006);
            const float _v1008 = __fmaf_rn(F4_r10, 0.0f, F4_t1);
            const float _v1009 = __fmaf_rn(F4_r11, 0.0f, _v1008);
            const float cb51_y = __fmaf_rn(F4_r12, 0.09000000357627869f, _v1009);
            const float _v1011 = __fmaf_rn(F4_r20, 0.0f, F4_t2);
            const float _v1012 = __fmaf_rn(F4_r21, 0.0f, _v1011);
            const float cb51_z = __fmaf_rn(F4_r22, 0.09000000357627869f, _v1012);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb51_x, cb51_y, cb51_z, 0.07000000029802322f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_11(F4_r00, F4_r01, F4_r02, F4_r10, F4_r11, F4_r12, F4_r20, F4_r21, F4_r22, F4_t0, F4_t1, F4_t2, sb);
                if (vg::self_cross<9, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. wrist_3_link
        {
            const float _v1014 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1015 = __fmaf_rn(F2_r01, 0.0f, _v1014);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1015);
            const float _v1017 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1018 = __fmaf_rn(F2_r11, 0.0f, _v1017);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1018);
            const float _v1020 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1021 = __fmaf_rn(0.0f, 0.0f, _v1020);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1021);
            const float _v1023 = __fmaf_rn(F5_r00, 0.0f, F5_t0);
            const float _v1024 = __fmaf_rn(F5_r01, 0.05999999865889549f, _v1023);
            const float cb50_x = __fmaf_rn(F5_r02, 0.0f, _v1024);
            const float _v1026 = __fmaf_rn(F5_r10, 0.0f, F5_t1);
            const float _v1027 = __fmaf_rn(F5_r11, 0.05999999865889549f, _v1026);
            const float cb50_y = __fmaf_rn(F5_r12, 0.0f, _v1027);
            const float _v1029 = __fmaf_rn(F5_r20, 0.0f, F5_t2);
            const float _v1030 = __fmaf_rn(F5_r21, 0.05999999865889549f, _v1029);
            const float cb50_z = __fmaf_rn(F5_r22, 0.0f, _v1030);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb50_x, cb50_y, cb50_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_10(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. fts_robotside
        {
            const float _v1032 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1033 = __fmaf_rn(F2_r01, 0.0f, _v1032);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1033);
            const float _v1035 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1036 = __fmaf_rn(F2_r11, 0.0f, _v1035);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1036);
            const float _v1038 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1039 = __fmaf_rn(0.0f, 0.0f, _v1038);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1039);
            const float _v1041 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
            const float _v1042 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v1041);
            const float cb49_x = __fmaf_rn(F5_r02, 0.0f, _v1042);
            const float _v1044 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
            const float _v1045 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v1044);
            const float cb49_y = __fmaf_rn(F5_r12, 0.0f, _v1045);
            const float _v1047 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
            const float _v1048 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v1047);
            const float cb49_z = __fmaf_rn(F5_r22, 0.0f, _v1048);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb49_x, cb49_y, cb49_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_9(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_base_link
        {
            const float _v1050 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1051 = __fmaf_rn(F2_r01, 0.0f, _v1050);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1051);
            const float _v1053 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1054 = __fmaf_rn(F2_r11, 0.0f, _v1053);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1054);
            const float _v1056 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1057 = __fmaf_rn(0.0f, 0.0f, _v1056);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1057);
            const float _v1059 = __fmaf_rn(F5_r00, -3.185292371199466e-05f, F5_t0);
            const float _v1060 = __fmaf_rn(F5_r01, 0.1572999805212021f, _v1059);
            const float cb48_x = __fmaf_rn(F5_r02, 0.0005318530602380633f, _v1060);
            const float _v1062 = __fmaf_rn(F5_r10, -3.185292371199466e-05f, F5_t1);
            const float _v1063 = __fmaf_rn(F5_r11, 0.1572999805212021f, _v1062);
            const float cb48_y = __fmaf_rn(F5_r12, 0.0005318530602380633f, _v1063);
            const float _v1065 = __fmaf_rn(F5_r20, -3.185292371199466e-05f, F5_t2);
            const float _v1066 = __fmaf_rn(F5_r21, 0.1572999805212021f, _v1065);
            const float cb48_z = __fmaf_rn(F5_r22, 0.0005318530602380633f, _v1066);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb48_x, cb48_y, cb48_z, 0.05999999865889549f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_8(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_left_inner_knuckle_link
        {
            const float _v1068 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1069 = __fmaf_rn(F2_r01, 0.0f, _v1068);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1069);
            const float _v1071 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1072 = __fmaf_rn(F2_r11, 0.0f, _v1071);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1072);
            const float _v1074 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1075 = __fmaf_rn(0.0f, 0.0f, _v1074);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1075);
            const float _v1077 = __fmaf_rn(F5_r00, 0.032628871500492096f, F5_t0);
            const float _v1078 = __fmaf_rn(F5_r01, 0.20663347840309143f, _v1077);
            const float cb47_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v1078);
            const float _v1080 = __fmaf_rn(F5_r10, 0.032628871500492096f, F5_t1);
            const float _v1081 = __fmaf_rn(F5_r11, 0.20663347840309143f, _v1080);
            const float cb47_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v1081);
            const float _v1083 = __fmaf_rn(F5_r20, 0.032628871500492096f, F5_t2);
            const float _v1084 = __fmaf_rn(F5_r21, 0.20663347840309143f, _v1083);
            const float cb47_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v1084);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb47_x, cb47_y, cb47_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_7(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_left_finger_tip_link
        {
            const float _v1086 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1087 = __fmaf_rn(F2_r01, 0.0f, _v1086);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1087);
            const float _v1089 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1090 = __fmaf_rn(F2_r11, 0.0f, _v1089);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1090);
            const float _v1092 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1093 = __fmaf_rn(0.0f, 0.0f, _v1092);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1093);
            const float _v1095 = __fmaf_rn(F5_r00, 0.047183919697999954f, F5_t0);
            const float _v1096 = __fmaf_rn(F5_r01, 0.24464209377765656f, _v1095);
            const float cb46_x = __fmaf_rn(F5_r02, 0.0006013759993948042f, _v1096);
            const float _v1098 = __fmaf_rn(F5_r10, 0.047183919697999954f, F5_t1);
            const float _v1099 = __fmaf_rn(F5_r11, 0.24464209377765656f, _v1098);
            const float cb46_y = __fmaf_rn(F5_r12, 0.0006013759993948042f, _v1099);
            const float _v1101 = __fmaf_rn(F5_r20, 0.047183919697999954f, F5_t2);
            const float _v1102 = __fmaf_rn(F5_r21, 0.24464209377765656f, _v1101);
            const float cb46_z = __fmaf_rn(F5_r22, 0.0006013759993948042f, _v1102);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb46_x, cb46_y, cb46_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_6(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_left_knuckle_link
        {
            const float _v1104 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1105 = __fmaf_rn(F2_r01, 0.0f, _v1104);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1105);
            const float _v1107 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1108 = __fmaf_rn(F2_r11, 0.0f, _v1107);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1108);
            const float _v1110 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1111 = __fmaf_rn(0.0f, 0.0f, _v1110);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1111);
            const float _v1113 = __fmaf_rn(F5_r00, 0.030551131814718246f, F5_t0);
            const float _v1114 = __fmaf_rn(F5_r01, 0.18011634051799774f, _v1113);
            const float cb45_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v1114);
            const float _v1116 = __fmaf_rn(F5_r10, 0.030551131814718246f, F5_t1);
            const float _v1117 = __fmaf_rn(F5_r11, 0.18011634051799774f, _v1116);
            const float cb45_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v1117);
            const float _v1119 = __fmaf_rn(F5_r20, 0.030551131814718246f, F5_t2);
            const float _v1120 = __fmaf_rn(F5_r21, 0.18011634051799774f, _v1119);
            const float cb45_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v1120);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb45_x, cb45_y, cb45_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_5(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_left_finger_link
        {
            const float _v1122 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1123 = __fmaf_rn(F2_r01, 0.0f, _v1122);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1123);
            const float _v1125 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1126 = __fmaf_rn(F2_r11, 0.0f, _v1125);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1126);
            const float _v1128 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1129 = __fmaf_rn(0.0f, 0.0f, _v1128);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1129);
            const float _v1131 = __fmaf_rn(F5_r00, 0.062227778136730194f, F5_t0);
            const float _v1132 = __fmaf_rn(F5_r01, 0.19820760190486908f, _v1131);
            const float cb44_x = __fmaf_rn(F5_r02, 0.0005643894546665251f, _v1132);
            const float _v1134 = __fmaf_rn(F5_r10, 0.062227778136730194f, F5_t1);
            const float _v1135 = __fmaf_rn(F5_r11, 0.19820760190486908f, _v1134);
            const float cb44_y = __fmaf_rn(F5_r12, 0.0005643894546665251f, _v1135);
            const float _v1137 = __fmaf_rn(F5_r20, 0.062227778136730194f, F5_t2);
            const float _v1138 = __fmaf_rn(F5_r21, 0.19820760190486908f, _v1137);
            const float cb44_z = __fmaf_rn(F5_r22, 0.0005643894546665251f, _v1138);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb44_x, cb44_y, cb44_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_4(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_right_inner_knuckle_link
        {
            const float _v1140 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1141 = __fmaf_rn(F2_r01, 0.0f, _v1140);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1141);
            const float _v1143 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1144 = __fmaf_rn(F2_r11, 0.0f, _v1143);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1144);
            const float _v1146 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1147 = __fmaf_rn(0.0f, 0.0f, _v1146);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1147);
            const float _v1149 = __fmaf_rn(F5_r00, -0.03277110680937767f, F5_t0);
            const float _v1150 = __fmaf_rn(F5_r01, 0.20658139884471893f, _v1149);
            const float cb43_x = __fmaf_rn(F5_r02, 0.0005711179692298174f, _v1150);
            const float _v1152 = __fmaf_rn(F5_r10, -0.03277110680937767f, F5_t1);
            const float _v1153 = __fmaf_rn(F5_r11, 0.20658139884471893f, _v1152);
            const float cb43_y = __fmaf_rn(F5_r12, 0.0005711179692298174f, _v1153);
            const float _v1155 = __fmaf_rn(F5_r20, -0.03277110680937767f, F5_t2);
            const float _v1156 = __fmaf_rn(F5_r21, 0.20658139884471893f, _v1155);
            const float cb43_z = __fmaf_rn(F5_r22, 0.0005711179692298174f, _v1156);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb43_x, cb43_y, cb43_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_3(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_right_finger_tip_link
        {
            const float _v1158 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1159 = __fmaf_rn(F2_r01, 0.0f, _v1158);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1159);
            const float _v1161 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1162 = __fmaf_rn(F2_r11, 0.0f, _v1161);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1162);
            const float _v1164 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1165 = __fmaf_rn(0.0f, 0.0f, _v1164);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1165);
            const float _v1167 = __fmaf_rn(F5_r00, -0.0469076968729496f, F5_t0);
            const float _v1168 = __fmaf_rn(F5_r01, 0.2449275404214859f, _v1167);
            const float cb42_x = __fmaf_rn(F5_r02, 0.0006016629631631076f, _v1168);
            const float _v1170 = __fmaf_rn(F5_r10, -0.0469076968729496f, F5_t1);
            const float _v1171 = __fmaf_rn(F5_r11, 0.2449275404214859f, _v1170);
            const float cb42_y = __fmaf_rn(F5_r12, 0.0006016629631631076f, _v1171);
            const float _v1173 = __fmaf_rn(F5_r20, -0.0469076968729496f, F5_t2);
            const float _v1174 = __fmaf_rn(F5_r21, 0.2449275404214859f, _v1173);
            const float cb42_z = __fmaf_rn(F5_r22, 0.0006016629631631076f, _v1174);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb42_x, cb42_y, cb42_z, 0.027499999850988388f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_2(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 2>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_right_knuckle_link
        {
            const float _v1176 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1177 = __fmaf_rn(F2_r01, 0.0f, _v1176);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1177);
            const float _v1179 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1180 = __fmaf_rn(F2_r11, 0.0f, _v1179);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1180);
            const float _v1182 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1183 = __fmaf_rn(0.0f, 0.0f, _v1182);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1183);
            const float _v1185 = __fmaf_rn(F5_r00, -0.030651137232780457f, F5_t0);
            const float _v1186 = __fmaf_rn(F5_r01, 0.18006761372089386f, _v1185);
            const float cb41_x = __fmaf_rn(F5_r02, 0.0005500029656104743f, _v1186);
            const float _v1188 = __fmaf_rn(F5_r10, -0.030651137232780457f, F5_t1);
            const float _v1189 = __fmaf_rn(F5_r11, 0.18006761372089386f, _v1188);
            const float cb41_y = __fmaf_rn(F5_r12, 0.0005500029656104743f, _v1189);
            const float _v1191 = __fmaf_rn(F5_r20, -0.030651137232780457f, F5_t2);
            const float _v1192 = __fmaf_rn(F5_r21, 0.18006761372089386f, _v1191);
            const float cb41_z = __fmaf_rn(F5_r22, 0.0005500029656104743f, _v1192);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb41_x, cb41_y, cb41_z, 0.019999999552965164f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_1(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 1>(ctx, sa, sb, need)) return;
            }
        }
        // self: forearm_link vs. robotiq_85_right_finger_link
        {
            const float _v1194 = __fmaf_rn(F2_r00, 0.0f, F2_t0);
            const float _v1195 = __fmaf_rn(F2_r01, 0.0f, _v1194);
            const float ca53_x = __fmaf_rn(F2_r02, 0.17000000178813934f, _v1195);
            const float _v1197 = __fmaf_rn(F2_r10, 0.0f, F2_t1);
            const float _v1198 = __fmaf_rn(F2_r11, 0.0f, _v1197);
            const float ca53_y = __fmaf_rn(F2_r12, 0.17000000178813934f, _v1198);
            const float _v1200 = __fmaf_rn(F2_r20, 0.0f, F2_t2);
            const float _v1201 = __fmaf_rn(0.0f, 0.0f, _v1200);
            const float ca53_z = __fmaf_rn(F2_r22, 0.17000000178813934f, _v1201);
            const float _v1203 = __fmaf_rn(F5_r00, -0.06237537041306496f, F5_t0);
            const float _v1204 = __fmaf_rn(F5_r01, 0.19844098389148712f, _v1203);
            const float cb40_x = __fmaf_rn(F5_r02, 0.0005646542995236814f, _v1204);
            const float _v1206 = __fmaf_rn(F5_r10, -0.06237537041306496f, F5_t1);
            const float _v1207 = __fmaf_rn(F5_r11, 0.19844098389148712f, _v1206);
            const float cb40_y = __fmaf_rn(F5_r12, 0.0005646542995236814f, _v1207);
            const float _v1209 = __fmaf_rn(F5_r20, -0.06237537041306496f, F5_t2);
            const float _v1210 = __fmaf_rn(F5_r21, 0.19844098389148712f, _v1209);
            const float cb40_z = __fmaf_rn(F5_r22, 0.0005646542995236814f, _v1210);
            const unsigned need = ctx.self_hit(ca53_x, ca53_y, ca53_z, 0.25f, cb40_x, cb40_y, cb40_z, 0.03500000014901161f, ctx.alive);
            if (need)
            {
                fine_13(F2_r00, F2_r01, F2_r02, F2_r10, F2_r11, F2_r12, F2_r20, F2_r22, F2_t0, F2_t1, F2_t2, sa);
                fine_0(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<9, 3>(ctx, sa, sb, need)) return;
            }
        }
        // self: wrist_1_link vs. fts_robotside
        {
            const float _v1212 = __fmaf_rn(F3_r00, 0.0f, F3_t0);
            const float _v1213 = __fmaf_rn(F3_r01, 0.09000000357627869f, _v1212);
            const float ca52_x = __fmaf_rn(F3_r02, 0.0f, _v1213);
            const float _v1215 = __fmaf_rn(F3_r10, 0.0f, F3_t1);
            const float _v1216 = __fmaf_rn(F3_r11, 0.09000000357627869f, _v1215);
            const float ca52_y = __fmaf_rn(F3_r12, 0.0f, _v1216);
            const float _v1218 = __fmaf_rn(F3_r20, 0.0f, F3_t2);
            const float _v1219 = __fmaf_rn(0.0f, 0.09000000357627869f, _v1218);
            const float ca52_z = __fmaf_rn(F3_r22, 0.0f, _v1219);
            const float _v1221 = __fmaf_rn(F5_r00, 1.5926561900414526e-05f, F5_t0);
            const float _v1222 = __fmaf_rn(F5_r01, 0.09730000793933868f, _v1221);
            const float cb49_x = __fmaf_rn(F5_r02, 0.0f, _v1222);
            const float _v1224 = __fmaf_rn(F5_r10, 1.5926561900414526e-05f, F5_t1);
            const float _v1225 = __fmaf_rn(F5_r11, 0.09730000793933868f, _v1224);
            const float cb49_y = __fmaf_rn(F5_r12, 0.0f, _v1225);
            const float _v1227 = __fmaf_rn(F5_r20, 1.5926561900414526e-05f, F5_t2);
            const float _v1228 = __fmaf_rn(F5_r21, 0.09730000793933868f, _v1227);
            const float cb49_z = __fmaf_rn(F5_r22, 0.0f, _v1228);
            const unsigned need = ctx.self_hit(ca52_x, ca52_y, ca52_z, 0.07000000029802322f, cb49_x, cb49_y, cb49_z, 0.03999999910593033f, ctx.alive);
            if (need)
            {
                fine_12(F3_r00, F3_r01, F3_r02, F3_r10, F3_r11, F3_r12, F3_r20, F3_r22, F3_t0, F3_t1, F3_t2, sa);
                fine_9(F5_r00, F5_r01, F5_r02, F5_r10, F5_r11, F5_r12, F5_r20, F5_r21, F5_r22, F5_t0, F5_t1, F5_t2, sb);
                if (vg::self_cross<3, 1>(ctx, sa, sb, need)) return;
            }
        }
    }
};
}  // namespace vg::robots
