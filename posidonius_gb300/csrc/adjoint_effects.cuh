// adjoint_effects.cuh -- GENERATED by posidonius_gb300/adjoint_codegen.py; do not edit.
//
// Per-planet additional-effect blocks (constant-time-lag tides, oblate
// flattening, Kidder 1995 general relativity) in the formulation of the FAST
// build, split for the implicit-midpoint loop: <block>_pre (once per half
// kick: position and tidal-parameter terms), <block>_iter (per iteration),
// the reverse sweeps <block>_iter_vjp / <block>_pre_vjp and the
// forward-mode (tangent) sweeps <block>_pre_jvp / <block>_iter_jvp.
#pragma once
#include <cmath>

#include "adjoint_blocks.cuh"

namespace posi_adj {

// adj_tides: pre inputs (x, y, z, sig_p, sig_h, k2_p, k2_h); iteration inputs (hv0, hv1, hv2, S0, S1, S2, H0, H1, H2, P0, P1, P2, Q0, Q1, Q2);
// constants (R, hR, hm, m)
constexpr int adj_tides_NPRE = 18;

// adj_tides: values fixed during a half kick (position, tidal parameters).
__host__ __device__ __forceinline__ void adj_tides_pre(double in_x, double in_y, double in_z, double in_sig_p, double in_sig_h, double in_k2_p, double in_k2_h,
        double c_R, double c_hR, double c_hm, double c_m, double* __restrict__ pre) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t33 = 1.0 / t23;
    const double t34 = in_x * t33;
    const double t35 = in_y * t33;
    const double t36 = in_z * t33;
    const double t62 = t23 * t23;
    const double t63 = t23 * t62;
    const double t64 = t62 * t62;
    const double t65 = t63 * t64;
    const double t66 = t23 * t65;
    const double t67 = c_m * c_m;
    const double t68 = c_hm * c_hm;
    const double t69 = c_hR * c_hR;
    const double t70 = t69 * t69;
    const double t71 = t70 * t70;
    const double t72 = t69 * t71;
    const double t73 = t67 * t72;
    const double t74 = in_sig_h * t73;
    const double t75 = c_R * c_R;
    const double t76 = t75 * t75;
    const double t77 = t76 * t76;
    const double t78 = t75 * t77;
    const double t79 = t68 * t78;
    const double t80 = in_sig_p * t79;
    const double t82 = t74 * 4.5;
    const double t83 = 1.0 / t65;
    const double t84 = t82 * t83;
    const double t85 = t80 * 4.5;
    const double t86 = t83 * t85;
    const double t89 = kK2 * -3.0;
    const double t90 = t83 * t89;
    const double t91 = c_hR * t70;
    const double t92 = t67 * t91;
    const double t93 = in_k2_h * t92;
    const double t94 = c_R * t76;
    const double t95 = t68 * t94;
    const double t96 = in_k2_p * t95;
    const double t97 = t93 + t96;
    const double t98 = t90 * t97;
    const double t99 = t33 * t84;
    const double t100 = t33 * t86;
    const double t102 = 1.0 / t66;
    const double t103 = -13.5 * t102;
    const double t105 = t74 + t80;
    const double t108 = t84 + t86;
    const double t109 = t33 * t108;
    const double t142 = 1.0 / c_m;
    const double t146 = t23 * t86;
    const double t147 = t23 * t84;
    pre[0] = in_x;
    pre[1] = in_y;
    pre[2] = in_z;
    pre[3] = t33;
    pre[4] = t103;
    pre[5] = t105;
    pre[6] = t98;
    pre[7] = t109;
    pre[8] = t99;
    pre[9] = t100;
    pre[10] = t34;
    pre[11] = t35;
    pre[12] = t36;
    pre[13] = t142;
    pre[14] = t86;
    pre[15] = t84;
    pre[16] = t146;
    pre[17] = t147;
}

// adj_tides: one midpoint iteration.  Outputs: a[3] (planet acceleration),
// dl[3] (planet dL/dt), th[3] (dL/dt of the host due to this planet).
__host__ __device__ __forceinline__ void adj_tides_iter(const double* __restrict__ pre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_R, double c_hR, double c_hm, double c_m, double* __restrict__ out) {
    const double t37 = pre[0] * in_hv0;
    const double t38 = pre[1] * in_hv1;
    const double t39 = t37 + t38;
    const double t40 = pre[2] * in_hv2;
    const double t41 = t39 + t40;
    const double t42 = pre[3] * t41;
    const double t43 = pre[0] * in_Q0;
    const double t44 = pre[1] * in_Q1;
    const double t45 = t43 + t44;
    const double t46 = pre[2] * in_Q2;
    const double t47 = t45 + t46;
    const double t48 = pre[0] * in_P0;
    const double t49 = pre[1] * in_P1;
    const double t50 = t48 + t49;
    const double t51 = pre[2] * in_P2;
    const double t52 = t50 + t51;
    const double t53 = pre[1] * in_hv2;
    const double t54 = pre[2] * in_hv1;
    const double t55 = t53 - t54;
    const double t56 = pre[2] * in_hv0;
    const double t57 = pre[0] * in_hv2;
    const double t58 = t56 - t57;
    const double t59 = pre[0] * in_hv1;
    const double t60 = pre[1] * in_hv0;
    const double t61 = t59 - t60;
    const double t104 = t42 * pre[4];
    const double t106 = t104 * pre[5];
    const double t107 = pre[6] + t106;
    const double t110 = t42 * pre[7];
    const double t111 = t107 + t110;
    const double t112 = in_H0 * pre[8];
    const double t113 = in_S0 * pre[9];
    const double t114 = t112 + t113;
    const double t115 = in_H1 * pre[8];
    const double t116 = in_S1 * pre[9];
    const double t117 = t115 + t116;
    const double t118 = in_H2 * pre[8];
    const double t119 = in_S2 * pre[9];
    const double t120 = t118 + t119;
    const double t121 = pre[2] * t117;
    const double t122 = pre[1] * t120;
    const double t123 = t121 - t122;
    const double t124 = pre[0] * t120;
    const double t125 = pre[2] * t114;
    const double t126 = t124 - t125;
    const double t127 = pre[1] * t114;
    const double t128 = pre[0] * t117;
    const double t129 = t127 - t128;
    const double t130 = pre[10] * t111;
    const double t131 = t123 + t130;
    const double t132 = in_hv0 * pre[7];
    const double t133 = t131 - t132;
    const double t134 = pre[11] * t111;
    const double t135 = t126 + t134;
    const double t136 = in_hv1 * pre[7];
    const double t137 = t135 - t136;
    const double t138 = pre[12] * t111;
    const double t139 = t129 + t138;
    const double t140 = in_hv2 * pre[7];
    const double t141 = t139 - t140;
    const double t143 = t133 * pre[13];
    const double t144 = t137 * pre[13];
    const double t145 = t141 * pre[13];
    const double t148 = t52 * pre[14];
    const double t149 = t47 * pre[15];
    const double t150 = in_S0 * pre[16];
    const double t151 = pre[10] * t148;
    const double t152 = t150 - t151;
    const double t153 = t55 * pre[9];
    const double t154 = t152 - t153;
    const double t155 = -t154;
    const double t156 = in_S1 * pre[16];
    const double t157 = pre[11] * t148;
    const double t158 = t156 - t157;
    const double t159 = t58 * pre[9];
    const double t160 = t158 - t159;
    const double t161 = -t160;
    const double t162 = in_S2 * pre[16];
    const double t163 = pre[12] * t148;
    const double t164 = t162 - t163;
    const double t165 = t61 * pre[9];
    const double t166 = t164 - t165;
    const double t167 = -t166;
    const double t168 = in_H0 * pre[17];
    const double t169 = pre[10] * t149;
    const double t170 = t168 - t169;
    const double t171 = t55 * pre[8];
    const double t172 = t170 - t171;
    const double t173 = -t172;
    const double t174 = in_H1 * pre[17];
    const double t175 = pre[11] * t149;
    const double t176 = t174 - t175;
    const double t177 = t58 * pre[8];
    const double t178 = t176 - t177;
    const double t179 = -t178;
    const double t180 = in_H2 * pre[17];
    const double t181 = pre[12] * t149;
    const double t182 = t180 - t181;
    const double t183 = t61 * pre[8];
    const double t184 = t182 - t183;
    const double t185 = -t184;
    out[0] = t143;
    out[1] = t144;
    out[2] = t145;
    out[3] = t155;
    out[4] = t161;
    out[5] = t167;
    out[6] = t173;
    out[7] = t179;
    out[8] = t185;
}

// adj_tides: VJP of one iteration.  bin[15] += adjoints of (hv0, hv1, hv2, S0, S1, S2, H0, H1, H2, P0, P1, P2, Q0, Q1, Q2);
// bpre[adj_tides_NPRE] += adjoints of the pre values.
__host__ __device__ __forceinline__ void adj_tides_iter_vjp(const double* __restrict__ pre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_R, double c_hR, double c_hm, double c_m, const double* __restrict__ bout, double* __restrict__ bin, double* __restrict__ bpre) {
    const double t37 = pre[0] * in_hv0;
    const double t38 = pre[1] * in_hv1;
    const double t39 = t37 + t38;
    const double t40 = pre[2] * in_hv2;
    const double t41 = t39 + t40;
    const double t42 = pre[3] * t41;
    const double t43 = pre[0] * in_Q0;
    const double t44 = pre[1] * in_Q1;
    const double t45 = t43 + t44;
    const double t46 = pre[2] * in_Q2;
    const double t47 = t45 + t46;
    const double t48 = pre[0] * in_P0;
    const double t49 = pre[1] * in_P1;
    const double t50 = t48 + t49;
    const double t51 = pre[2] * in_P2;
    const double t52 = t50 + t51;
    const double t53 = pre[1] * in_hv2;
    const double t54 = pre[2] * in_hv1;
    const double t55 = t53 - t54;
    const double t56 = pre[2] * in_hv0;
    const double t57 = pre[0] * in_hv2;
    const double t58 = t56 - t57;
    const double t59 = pre[0] * in_hv1;
    const double t60 = pre[1] * in_hv0;
    const double t61 = t59 - t60;
    const double t104 = t42 * pre[4];
    const double t106 = t104 * pre[5];
    const double t107 = pre[6] + t106;
    const double t110 = t42 * pre[7];
    const double t111 = t107 + t110;
    const double t112 = in_H0 * pre[8];
    const double t113 = in_S0 * pre[9];
    const double t114 = t112 + t113;
    const double t115 = in_H1 * pre[8];
    const double t116 = in_S1 * pre[9];
    const double t117 = t115 + t116;
    const double t118 = in_H2 * pre[8];
    const double t119 = in_S2 * pre[9];
    const double t120 = t118 + t119;
    const double t121 = pre[2] * t117;
    const double t122 = pre[1] * t120;
    const double t123 = t121 - t122;
    const double t124 = pre[0] * t120;
    const double t125 = pre[2] * t114;
    const double t126 = t124 - t125;
    const double t127 = pre[1] * t114;
    const double t128 = pre[0] * t117;
    const double t129 = t127 - t128;
    const double t130 = pre[10] * t111;
    const double t131 = t123 + t130;
    const double t132 = in_hv0 * pre[7];
    const double t133 = t131 - t132;
    const double t134 = pre[11] * t111;
    const double t135 = t126 + t134;
    const double t136 = in_hv1 * pre[7];
    const double t137 = t135 - t136;
    const double t138 = pre[12] * t111;
    const double t139 = t129 + t138;
    const double t140 = in_hv2 * pre[7];
    const double t141 = t139 - t140;
    const double t143 = t133 * pre[13];
    const double t144 = t137 * pre[13];
    const double t145 = t141 * pre[13];
    const double t148 = t52 * pre[14];
    const double t149 = t47 * pre[15];
    const double t150 = in_S0 * pre[16];
    const double t151 = pre[10] * t148;
    const double t152 = t150 - t151;
    const double t153 = t55 * pre[9];
    const double t154 = t152 - t153;
    const double t155 = -t154;
    const double t156 = in_S1 * pre[16];
    const double t157 = pre[11] * t148;
    const double t158 = t156 - t157;
    const double t159 = t58 * pre[9];
    const double t160 = t158 - t159;
    const double t161 = -t160;
    const double t162 = in_S2 * pre[16];
    const double t163 = pre[12] * t148;
    const double t164 = t162 - t163;
    const double t165 = t61 * pre[9];
    const double t166 = t164 - t165;
    const double t167 = -t166;
    const double t168 = in_H0 * pre[17];
    const double t169 = pre[10] * t149;
    const double t170 = t168 - t169;
    const double t171 = t55 * pre[8];
    const double t172 = t170 - t171;
    const double t173 = -t172;
    const double t174 = in_H1 * pre[17];
    const double t175 = pre[11] * t149;
    const double t176 = t174 - t175;
    const double t177 = t58 * pre[8];
    const double t178 = t176 - t177;
    const double t179 = -t178;
    const double t180 = in_H2 * pre[17];
    const double t181 = pre[12] * t149;
    const double t182 = t180 - t181;
    const double t183 = t61 * pre[8];
    const double t184 = t182 - t183;
    const double t185 = -t184;
    double b143 = bout[0];
    double b144 = bout[1];
    double b145 = bout[2];
    double b155 = bout[3];
    double b161 = bout[4];
    double b167 = bout[5];
    double b173 = bout[6];
    double b179 = bout[7];
    double b185 = bout[8];
    double b184 = -b185;
    double b182 = b184;
    double b183 = -b184;
    double b61 = b183 * pre[8];
    bpre[8] += b183 * t61;
    double b180 = b182;
    double b181 = -b182;
    bpre[12] += b181 * t149;
    double b149 = b181 * pre[12];
    double b_H2 = b180 * pre[17];
    bpre[17] += b180 * in_H2;
    double b178 = -b179;
    double b176 = b178;
    double b177 = -b178;
    double b58 = b177 * pre[8];
    bpre[8] += b177 * t58;
    double b174 = b176;
    double b175 = -b176;
    bpre[11] += b175 * t149;
    b149 += b175 * pre[11];
    double b_H1 = b174 * pre[17];
    bpre[17] += b174 * in_H1;
    double b172 = -b173;
    double b170 = b172;
    double b171 = -b172;
    double b55 = b171 * pre[8];
    bpre[8] += b171 * t55;
    double b168 = b170;
    double b169 = -b170;
    bpre[10] += b169 * t149;
    b149 += b169 * pre[10];
    double b_H0 = b168 * pre[17];
    bpre[17] += b168 * in_H0;
    double b166 = -b167;
    double b164 = b166;
    double b165 = -b166;
    b61 += b165 * pre[9];
    bpre[9] += b165 * t61;
    double b162 = b164;
    double b163 = -b164;
    bpre[12] += b163 * t148;
    double b148 = b163 * pre[12];
    double b_S2 = b162 * pre[16];
    bpre[16] += b162 * in_S2;
    double b160 = -b161;
    double b158 = b160;
    double b159 = -b160;
    b58 += b159 * pre[9];
    bpre[9] += b159 * t58;
    double b156 = b158;
    double b157 = -b158;
    bpre[11] += b157 * t148;
    b148 += b157 * pre[11];
    double b_S1 = b156 * pre[16];
    bpre[16] += b156 * in_S1;
    double b154 = -b155;
    double b152 = b154;
    double b153 = -b154;
    b55 += b153 * pre[9];
    bpre[9] += b153 * t55;
    double b150 = b152;
    double b151 = -b152;
    bpre[10] += b151 * t148;
    b148 += b151 * pre[10];
    double b_S0 = b150 * pre[16];
    bpre[16] += b150 * in_S0;
    double b47 = b149 * pre[15];
    bpre[15] += b149 * t47;
    double b52 = b148 * pre[14];
    bpre[14] += b148 * t52;
    double b141 = b145 * pre[13];
    double b137 = b144 * pre[13];
    double b133 = b143 * pre[13];
    double b139 = b141;
    double b140 = -b141;
    double b_hv2 = b140 * pre[7];
    bpre[7] += b140 * in_hv2;
    double b129 = b139;
    double b138 = b139;
    bpre[12] += b138 * t111;
    double b111 = b138 * pre[12];
    double b135 = b137;
    double b136 = -b137;
    double b_hv1 = b136 * pre[7];
    bpre[7] += b136 * in_hv1;
    double b126 = b135;
    double b134 = b135;
    bpre[11] += b134 * t111;
    b111 += b134 * pre[11];
    double b131 = b133;
    double b132 = -b133;
    double b_hv0 = b132 * pre[7];
    bpre[7] += b132 * in_hv0;
    double b123 = b131;
    double b130 = b131;
    bpre[10] += b130 * t111;
    b111 += b130 * pre[10];
    double b127 = b129;
    double b128 = -b129;
    bpre[0] += b128 * t117;
    double b117 = b128 * pre[0];
    bpre[1] += b127 * t114;
    double b114 = b127 * pre[1];
    double b124 = b126;
    double b125 = -b126;
    bpre[2] += b125 * t114;
    b114 += b125 * pre[2];
    bpre[0] += b124 * t120;
    double b120 = b124 * pre[0];
    double b121 = b123;
    double b122 = -b123;
    bpre[1] += b122 * t120;
    b120 += b122 * pre[1];
    bpre[2] += b121 * t117;
    b117 += b121 * pre[2];
    double b118 = b120;
    double b119 = b120;
    b_S2 += b119 * pre[9];
    bpre[9] += b119 * in_S2;
    b_H2 += b118 * pre[8];
    bpre[8] += b118 * in_H2;
    double b115 = b117;
    double b116 = b117;
    b_S1 += b116 * pre[9];
    bpre[9] += b116 * in_S1;
    b_H1 += b115 * pre[8];
    bpre[8] += b115 * in_H1;
    double b112 = b114;
    double b113 = b114;
    b_S0 += b113 * pre[9];
    bpre[9] += b113 * in_S0;
    b_H0 += b112 * pre[8];
    bpre[8] += b112 * in_H0;
    double b107 = b111;
    double b110 = b111;
    double b42 = b110 * pre[7];
    bpre[7] += b110 * t42;
    bpre[6] += b107;
    double b106 = b107;
    double b104 = b106 * pre[5];
    bpre[5] += b106 * t104;
    b42 += b104 * pre[4];
    bpre[4] += b104 * t42;
    double b59 = b61;
    double b60 = -b61;
    bpre[1] += b60 * in_hv0;
    b_hv0 += b60 * pre[1];
    bpre[0] += b59 * in_hv1;
    b_hv1 += b59 * pre[0];
    double b56 = b58;
    double b57 = -b58;
    bpre[0] += b57 * in_hv2;
    b_hv2 += b57 * pre[0];
    bpre[2] += b56 * in_hv0;
    b_hv0 += b56 * pre[2];
    double b53 = b55;
    double b54 = -b55;
    bpre[2] += b54 * in_hv1;
    b_hv1 += b54 * pre[2];
    bpre[1] += b53 * in_hv2;
    b_hv2 += b53 * pre[1];
    double b50 = b52;
    double b51 = b52;
    bpre[2] += b51 * in_P2;
    double b_P2 = b51 * pre[2];
    double b48 = b50;
    double b49 = b50;
    bpre[1] += b49 * in_P1;
    double b_P1 = b49 * pre[1];
    bpre[0] += b48 * in_P0;
    double b_P0 = b48 * pre[0];
    double b45 = b47;
    double b46 = b47;
    bpre[2] += b46 * in_Q2;
    double b_Q2 = b46 * pre[2];
    double b43 = b45;
    double b44 = b45;
    bpre[1] += b44 * in_Q1;
    double b_Q1 = b44 * pre[1];
    bpre[0] += b43 * in_Q0;
    double b_Q0 = b43 * pre[0];
    bpre[3] += b42 * t41;
    double b41 = b42 * pre[3];
    double b39 = b41;
    double b40 = b41;
    bpre[2] += b40 * in_hv2;
    b_hv2 += b40 * pre[2];
    double b37 = b39;
    double b38 = b39;
    bpre[1] += b38 * in_hv1;
    b_hv1 += b38 * pre[1];
    bpre[0] += b37 * in_hv0;
    b_hv0 += b37 * pre[0];
    bin[0] += b_hv0;
    bin[1] += b_hv1;
    bin[2] += b_hv2;
    bin[3] += b_S0;
    bin[4] += b_S1;
    bin[5] += b_S2;
    bin[6] += b_H0;
    bin[7] += b_H1;
    bin[8] += b_H2;
    bin[9] += b_P0;
    bin[10] += b_P1;
    bin[11] += b_P2;
    bin[12] += b_Q0;
    bin[13] += b_Q1;
    bin[14] += b_Q2;
}

// adj_tides: VJP of the pre values.  bin[7] += adjoints of (x, y, z, sig_p, sig_h, k2_p, k2_h).
__host__ __device__ __forceinline__ void adj_tides_pre_vjp(double in_x, double in_y, double in_z, double in_sig_p, double in_sig_h, double in_k2_p, double in_k2_h,
        double c_R, double c_hR, double c_hm, double c_m, const double* __restrict__ bpre, double* __restrict__ bin) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t33 = 1.0 / t23;
    const double t34 = in_x * t33;
    const double t35 = in_y * t33;
    const double t36 = in_z * t33;
    const double t62 = t23 * t23;
    const double t63 = t23 * t62;
    const double t64 = t62 * t62;
    const double t65 = t63 * t64;
    const double t66 = t23 * t65;
    const double t67 = c_m * c_m;
    const double t68 = c_hm * c_hm;
    const double t69 = c_hR * c_hR;
    const double t70 = t69 * t69;
    const double t71 = t70 * t70;
    const double t72 = t69 * t71;
    const double t73 = t67 * t72;
    const double t74 = in_sig_h * t73;
    const double t75 = c_R * c_R;
    const double t76 = t75 * t75;
    const double t77 = t76 * t76;
    const double t78 = t75 * t77;
    const double t79 = t68 * t78;
    const double t80 = in_sig_p * t79;
    const double t82 = t74 * 4.5;
    const double t83 = 1.0 / t65;
    const double t84 = t82 * t83;
    const double t85 = t80 * 4.5;
    const double t86 = t83 * t85;
    const double t89 = kK2 * -3.0;
    const double t90 = t83 * t89;
    const double t91 = c_hR * t70;
    const double t92 = t67 * t91;
    const double t93 = in_k2_h * t92;
    const double t94 = c_R * t76;
    const double t95 = t68 * t94;
    const double t96 = in_k2_p * t95;
    const double t97 = t93 + t96;
    const double t98 = t90 * t97;
    const double t99 = t33 * t84;
    const double t100 = t33 * t86;
    const double t102 = 1.0 / t66;
    const double t103 = -13.5 * t102;
    const double t105 = t74 + t80;
    const double t108 = t84 + t86;
    const double t109 = t33 * t108;
    const double t142 = 1.0 / c_m;
    const double t146 = t23 * t86;
    const double t147 = t23 * t84;
    double b_x = bpre[0];
    double b_y = bpre[1];
    double b_z = bpre[2];
    double b33 = bpre[3];
    double b103 = bpre[4];
    double b105 = bpre[5];
    double b98 = bpre[6];
    double b109 = bpre[7];
    double b99 = bpre[8];
    double b100 = bpre[9];
    double b34 = bpre[10];
    double b35 = bpre[11];
    double b36 = bpre[12];
    double b86 = bpre[14];
    double b84 = bpre[15];
    double b146 = bpre[16];
    double b147 = bpre[17];
    double b23 = b147 * t84;
    b84 += b147 * t23;
    b23 += b146 * t86;
    b86 += b146 * t23;
    b33 += b109 * t108;
    double b108 = b109 * t33;
    b84 += b108;
    b86 += b108;
    double b74 = b105;
    double b80 = b105;
    double b102 = b103 * -13.5;
    double b66 = -b102 * t102 * t102;
    b33 += b100 * t86;
    b86 += b100 * t33;
    b33 += b99 * t84;
    b84 += b99 * t33;
    double b90 = b98 * t97;
    double b97 = b98 * t90;
    double b93 = b97;
    double b96 = b97;
    double b_k2_p = b96 * t95;
    double b_k2_h = b93 * t92;
    double b83 = b90 * t89;
    b83 += b86 * t85;
    double b85 = b86 * t83;
    b80 += b85 * 4.5;
    double b82 = b84 * t83;
    b83 += b84 * t82;
    double b65 = -b83 * t83 * t83;
    b74 += b82 * 4.5;
    double b_sig_p = b80 * t79;
    double b_sig_h = b74 * t73;
    b23 += b66 * t65;
    b65 += b66 * t23;
    double b63 = b65 * t64;
    double b64 = b65 * t63;
    double b62 = 2.0 * b64 * t62;
    b23 += b63 * t62;
    b62 += b63 * t23;
    b23 += 2.0 * b62 * t23;
    b_z += b36 * t33;
    b33 += b36 * in_z;
    b_y += b35 * t33;
    b33 += b35 * in_y;
    b_x += b34 * t33;
    b33 += b34 * in_x;
    b23 += -b33 * t33 * t33;
    double b22 = 0.5 * b23 / t23;
    double b20 = b22;
    double b21 = b22;
    b_z += 2.0 * b21 * in_z;
    double b18 = b20;
    double b19 = b20;
    b_y += 2.0 * b19 * in_y;
    b_x += 2.0 * b18 * in_x;
    bin[0] += b_x;
    bin[1] += b_y;
    bin[2] += b_z;
    bin[3] += b_sig_p;
    bin[4] += b_sig_h;
    bin[5] += b_k2_p;
    bin[6] += b_k2_h;
}

// adj_tides: pre values and their tangents (din[i * NT + k]: tangent k of pre input i).
template <int NT>
__host__ __device__ __forceinline__ void adj_tides_pre_jvp(double in_x, double in_y, double in_z, double in_sig_p, double in_sig_h, double in_k2_p, double in_k2_h,
        double c_R, double c_hR, double c_hm, double c_m, const double* __restrict__ din, double* __restrict__ pre,
        double* __restrict__ dpre) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t33 = 1.0 / t23;
    const double t34 = in_x * t33;
    const double t35 = in_y * t33;
    const double t36 = in_z * t33;
    const double t62 = t23 * t23;
    const double t63 = t23 * t62;
    const double t64 = t62 * t62;
    const double t65 = t63 * t64;
    const double t66 = t23 * t65;
    const double t67 = c_m * c_m;
    const double t68 = c_hm * c_hm;
    const double t69 = c_hR * c_hR;
    const double t70 = t69 * t69;
    const double t71 = t70 * t70;
    const double t72 = t69 * t71;
    const double t73 = t67 * t72;
    const double t74 = in_sig_h * t73;
    const double t75 = c_R * c_R;
    const double t76 = t75 * t75;
    const double t77 = t76 * t76;
    const double t78 = t75 * t77;
    const double t79 = t68 * t78;
    const double t80 = in_sig_p * t79;
    const double t82 = t74 * 4.5;
    const double t83 = 1.0 / t65;
    const double t84 = t82 * t83;
    const double t85 = t80 * 4.5;
    const double t86 = t83 * t85;
    const double t89 = kK2 * -3.0;
    const double t90 = t83 * t89;
    const double t91 = c_hR * t70;
    const double t92 = t67 * t91;
    const double t93 = in_k2_h * t92;
    const double t94 = c_R * t76;
    const double t95 = t68 * t94;
    const double t96 = in_k2_p * t95;
    const double t97 = t93 + t96;
    const double t98 = t90 * t97;
    const double t99 = t33 * t84;
    const double t100 = t33 * t86;
    const double t102 = 1.0 / t66;
    const double t103 = -13.5 * t102;
    const double t105 = t74 + t80;
    const double t108 = t84 + t86;
    const double t109 = t33 * t108;
    const double t142 = 1.0 / c_m;
    const double t146 = t23 * t86;
    const double t147 = t23 * t84;
    double d18[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d18[k] = 2.0 * in_x * din[0 * NT + k];
    double d19[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d19[k] = 2.0 * in_y * din[1 * NT + k];
    double d20[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d20[k] = d18[k] + d19[k];
    double d21[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d21[k] = 2.0 * in_z * din[2 * NT + k];
    double d22[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d22[k] = d20[k] + d21[k];
    double d23[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d23[k] = 0.5 * d22[k] / t23;
    double d33[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d33[k] = -t33 * t33 * d23[k];
    double d34[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d34[k] = din[0 * NT + k] * t33 + in_x * d33[k];
    double d35[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d35[k] = din[1 * NT + k] * t33 + in_y * d33[k];
    double d36[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d36[k] = din[2 * NT + k] * t33 + in_z * d33[k];
    double d62[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d62[k] = 2.0 * t23 * d23[k];
    double d63[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d63[k] = d23[k] * t62 + t23 * d62[k];
    double d64[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d64[k] = 2.0 * t62 * d62[k];
    double d65[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d65[k] = d63[k] * t64 + t63 * d64[k];
    double d66[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d66[k] = d23[k] * t65 + t23 * d65[k];
    double d74[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d74[k] = din[4 * NT + k] * t73;
    double d80[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d80[k] = din[3 * NT + k] * t79;
    double d82[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d82[k] = d74[k] * 4.5;
    double d83[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d83[k] = -t83 * t83 * d65[k];
    double d84[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d84[k] = d82[k] * t83 + t82 * d83[k];
    double d85[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d85[k] = d80[k] * 4.5;
    double d86[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d86[k] = d83[k] * t85 + t83 * d85[k];
    double d90[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d90[k] = d83[k] * t89;
    double d93[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d93[k] = din[6 * NT + k] * t92;
    double d96[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d96[k] = din[5 * NT + k] * t95;
    double d97[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d97[k] = d93[k] + d96[k];
    double d98[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d98[k] = d90[k] * t97 + t90 * d97[k];
    double d99[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d99[k] = d33[k] * t84 + t33 * d84[k];
    double d100[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d100[k] = d33[k] * t86 + t33 * d86[k];
    double d102[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d102[k] = -t102 * t102 * d66[k];
    double d103[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d103[k] = -13.5 * d102[k];
    double d105[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d105[k] = d74[k] + d80[k];
    double d108[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d108[k] = d84[k] + d86[k];
    double d109[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d109[k] = d33[k] * t108 + t33 * d108[k];
    double d146[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d146[k] = d23[k] * t86 + t23 * d86[k];
    double d147[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d147[k] = d23[k] * t84 + t23 * d84[k];
    pre[0] = in_x;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[0 * NT + k] = din[0 * NT + k];
    pre[1] = in_y;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[1 * NT + k] = din[1 * NT + k];
    pre[2] = in_z;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[2 * NT + k] = din[2 * NT + k];
    pre[3] = t33;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[3 * NT + k] = d33[k];
    pre[4] = t103;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[4 * NT + k] = d103[k];
    pre[5] = t105;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[5 * NT + k] = d105[k];
    pre[6] = t98;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[6 * NT + k] = d98[k];
    pre[7] = t109;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[7 * NT + k] = d109[k];
    pre[8] = t99;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[8 * NT + k] = d99[k];
    pre[9] = t100;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[9 * NT + k] = d100[k];
    pre[10] = t34;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[10 * NT + k] = d34[k];
    pre[11] = t35;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[11 * NT + k] = d35[k];
    pre[12] = t36;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[12 * NT + k] = d36[k];
    pre[13] = t142;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[13 * NT + k] = 0.0;
    pre[14] = t86;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[14 * NT + k] = d86[k];
    pre[15] = t84;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[15 * NT + k] = d84[k];
    pre[16] = t146;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[16 * NT + k] = d146[k];
    pre[17] = t147;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[17 * NT + k] = d147[k];
}

// adj_tides: one iteration, outputs and their tangents (din[i * NT + k] for the
// iteration inputs; dout[o * NT + k]).
template <int NT>
__host__ __device__ __forceinline__ void adj_tides_iter_jvp(const double* __restrict__ pre,
        const double* __restrict__ dpre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_R, double c_hR, double c_hm, double c_m, const double* __restrict__ din, double* __restrict__ out,
        double* __restrict__ dout) {
    const double t37 = pre[0] * in_hv0;
    const double t38 = pre[1] * in_hv1;
    const double t39 = t37 + t38;
    const double t40 = pre[2] * in_hv2;
    const double t41 = t39 + t40;
    const double t42 = pre[3] * t41;
    const double t43 = pre[0] * in_Q0;
    const double t44 = pre[1] * in_Q1;
    const double t45 = t43 + t44;
    const double t46 = pre[2] * in_Q2;
    const double t47 = t45 + t46;
    const double t48 = pre[0] * in_P0;
    const double t49 = pre[1] * in_P1;
    const double t50 = t48 + t49;
    const double t51 = pre[2] * in_P2;
    const double t52 = t50 + t51;
    const double t53 = pre[1] * in_hv2;
    const double t54 = pre[2] * in_hv1;
    const double t55 = t53 - t54;
    const double t56 = pre[2] * in_hv0;
    const double t57 = pre[0] * in_hv2;
    const double t58 = t56 - t57;
    const double t59 = pre[0] * in_hv1;
    const double t60 = pre[1] * in_hv0;
    const double t61 = t59 - t60;
    const double t104 = t42 * pre[4];
    const double t106 = t104 * pre[5];
    const double t107 = pre[6] + t106;
    const double t110 = t42 * pre[7];
    const double t111 = t107 + t110;
    const double t112 = in_H0 * pre[8];
    const double t113 = in_S0 * pre[9];
    const double t114 = t112 + t113;
    const double t115 = in_H1 * pre[8];
    const double t116 = in_S1 * pre[9];
    const double t117 = t115 + t116;
    const double t118 = in_H2 * pre[8];
    const double t119 = in_S2 * pre[9];
    const double t120 = t118 + t119;
    const double t121 = pre[2] * t117;
    const double t122 = pre[1] * t120;
    const double t123 = t121 - t122;
    const double t124 = pre[0] * t120;
    const double t125 = pre[2] * t114;
    const double t126 = t124 - t125;
    const double t127 = pre[1] * t114;
    const double t128 = pre[0] * t117;
    const double t129 = t127 - t128;
    const double t130 = pre[10] * t111;
    const double t131 = t123 + t130;
    const double t132 = in_hv0 * pre[7];
    const double t133 = t131 - t132;
    const double t134 = pre[11] * t111;
    const double t135 = t126 + t134;
    const double t136 = in_hv1 * pre[7];
    const double t137 = t135 - t136;
    const double t138 = pre[12] * t111;
    const double t139 = t129 + t138;
    const double t140 = in_hv2 * pre[7];
    const double t141 = t139 - t140;
    const double t143 = t133 * pre[13];
    const double t144 = t137 * pre[13];
    const double t145 = t141 * pre[13];
    const double t148 = t52 * pre[14];
    const double t149 = t47 * pre[15];
    const double t150 = in_S0 * pre[16];
    const double t151 = pre[10] * t148;
    const double t152 = t150 - t151;
    const double t153 = t55 * pre[9];
    const double t154 = t152 - t153;
    const double t155 = -t154;
    const double t156 = in_S1 * pre[16];
    const double t157 = pre[11] * t148;
    const double t158 = t156 - t157;
    const double t159 = t58 * pre[9];
    const double t160 = t158 - t159;
    const double t161 = -t160;
    const double t162 = in_S2 * pre[16];
    const double t163 = pre[12] * t148;
    const double t164 = t162 - t163;
    const double t165 = t61 * pre[9];
    const double t166 = t164 - t165;
    const double t167 = -t166;
    const double t168 = in_H0 * pre[17];
    const double t169 = pre[10] * t149;
    const double t170 = t168 - t169;
    const double t171 = t55 * pre[8];
    const double t172 = t170 - t171;
    const double t173 = -t172;
    const double t174 = in_H1 * pre[17];
    const double t175 = pre[11] * t149;
    const double t176 = t174 - t175;
    const double t177 = t58 * pre[8];
    const double t178 = t176 - t177;
    const double t179 = -t178;
    const double t180 = in_H2 * pre[17];
    const double t181 = pre[12] * t149;
    const double t182 = t180 - t181;
    const double t183 = t61 * pre[8];
    const double t184 = t182 - t183;
    const double t185 = -t184;
    double d37[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d37[k] = dpre[0 * NT + k] * in_hv0 + pre[0] * din[0 * NT + k];
    double d38[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d38[k] = dpre[1 * NT + k] * in_hv1 + pre[1] * din[1 * NT + k];
    double d39[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d39[k] = d37[k] + d38[k];
    double d40[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d40[k] = dpre[2 * NT + k] * in_hv2 + pre[2] * din[2 * NT + k];
    double d41[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d41[k] = d39[k] + d40[k];
    double d42[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d42[k] = dpre[3 * NT + k] * t41 + pre[3] * d41[k];
    double d43[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d43[k] = dpre[0 * NT + k] * in_Q0 + pre[0] * din[12 * NT + k];
    double d44[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d44[k] = dpre[1 * NT + k] * in_Q1 + pre[1] * din[13 * NT + k];
    double d45[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d45[k] = d43[k] + d44[k];
    double d46[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d46[k] = dpre[2 * NT + k] * in_Q2 + pre[2] * din[14 * NT + k];
    double d47[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d47[k] = d45[k] + d46[k];
    double d48[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d48[k] = dpre[0 * NT + k] * in_P0 + pre[0] * din[9 * NT + k];
    double d49[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d49[k] = dpre[1 * NT + k] * in_P1 + pre[1] * din[10 * NT + k];
    double d50[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d50[k] = d48[k] + d49[k];
    double d51[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d51[k] = dpre[2 * NT + k] * in_P2 + pre[2] * din[11 * NT + k];
    double d52[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d52[k] = d50[k] + d51[k];
    double d53[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d53[k] = dpre[1 * NT + k] * in_hv2 + pre[1] * din[2 * NT + k];
    double d54[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d54[k] = dpre[2 * NT + k] * in_hv1 + pre[2] * din[1 * NT + k];
    double d55[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d55[k] = d53[k] - d54[k];
    double d56[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d56[k] = dpre[2 * NT + k] * in_hv0 + pre[2] * din[0 * NT + k];
    double d57[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d57[k] = dpre[0 * NT + k] * in_hv2 + pre[0] * din[2 * NT + k];
    double d58[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d58[k] = d56[k] - d57[k];
    double d59[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d59[k] = dpre[0 * NT + k] * in_hv1 + pre[0] * din[1 * NT + k];
    double d60[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d60[k] = dpre[1 * NT + k] * in_hv0 + pre[1] * din[0 * NT + k];
    double d61[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d61[k] = d59[k] - d60[k];
    double d104[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d104[k] = d42[k] * pre[4] + t42 * dpre[4 * NT + k];
    double d106[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d106[k] = d104[k] * pre[5] + t104 * dpre[5 * NT + k];
    double d107[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d107[k] = dpre[6 * NT + k] + d106[k];
    double d110[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d110[k] = d42[k] * pre[7] + t42 * dpre[7 * NT + k];
    double d111[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d111[k] = d107[k] + d110[k];
    double d112[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d112[k] = din[6 * NT + k] * pre[8] + in_H0 * dpre[8 * NT + k];
    double d113[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d113[k] = din[3 * NT + k] * pre[9] + in_S0 * dpre[9 * NT + k];
    double d114[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d114[k] = d112[k] + d113[k];
    double d115[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d115[k] = din[7 * NT + k] * pre[8] + in_H1 * dpre[8 * NT + k];
    double d116[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d116[k] = din[4 * NT + k] * pre[9] + in_S1 * dpre[9 * NT + k];
    double d117[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d117[k] = d115[k] + d116[k];
    double d118[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d118[k] = din[8 * NT + k] * pre[8] + in_H2 * dpre[8 * NT + k];
    double d119[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d119[k] = din[5 * NT + k] * pre[9] + in_S2 * dpre[9 * NT + k];
    double d120[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d120[k] = d118[k] + d119[k];
    double d121[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d121[k] = dpre[2 * NT + k] * t117 + pre[2] * d117[k];
    double d122[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d122[k] = dpre[1 * NT + k] * t120 + pre[1] * d120[k];
    double d123[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d123[k] = d121[k] - d122[k];
    double d124[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d124[k] = dpre[0 * NT + k] * t120 + pre[0] * d120[k];
    double d125[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d125[k] = dpre[2 * NT + k] * t114 + pre[2] * d114[k];
    double d126[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d126[k] = d124[k] - d125[k];
    double d127[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d127[k] = dpre[1 * NT + k] * t114 + pre[1] * d114[k];
    double d128[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d128[k] = dpre[0 * NT + k] * t117 + pre[0] * d117[k];
    double d129[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d129[k] = d127[k] - d128[k];
    double d130[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d130[k] = dpre[10 * NT + k] * t111 + pre[10] * d111[k];
    double d131[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d131[k] = d123[k] + d130[k];
    double d132[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d132[k] = din[0 * NT + k] * pre[7] + in_hv0 * dpre[7 * NT + k];
    double d133[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d133[k] = d131[k] - d132[k];
    double d134[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d134[k] = dpre[11 * NT + k] * t111 + pre[11] * d111[k];
    double d135[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d135[k] = d126[k] + d134[k];
    double d136[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d136[k] = din[1 * NT + k] * pre[7] + in_hv1 * dpre[7 * NT + k];
    double d137[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d137[k] = d135[k] - d136[k];
    double d138[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d138[k] = dpre[12 * NT + k] * t111 + pre[12] * d111[k];
    double d139[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d139[k] = d129[k] + d138[k];
    double d140[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d140[k] = din[2 * NT + k] * pre[7] + in_hv2 * dpre[7 * NT + k];
    double d141[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d141[k] = d139[k] - d140[k];
    double d143[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d143[k] = d133[k] * pre[13];
    double d144[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d144[k] = d137[k] * pre[13];
    double d145[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d145[k] = d141[k] * pre[13];
    double d148[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d148[k] = d52[k] * pre[14] + t52 * dpre[14 * NT + k];
    double d149[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d149[k] = d47[k] * pre[15] + t47 * dpre[15 * NT + k];
    double d150[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d150[k] = din[3 * NT + k] * pre[16] + in_S0 * dpre[16 * NT + k];
    double d151[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d151[k] = dpre[10 * NT + k] * t148 + pre[10] * d148[k];
    double d152[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d152[k] = d150[k] - d151[k];
    double d153[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d153[k] = d55[k] * pre[9] + t55 * dpre[9 * NT + k];
    double d154[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d154[k] = d152[k] - d153[k];
    double d155[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d155[k] = -d154[k];
    double d156[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d156[k] = din[4 * NT + k] * pre[16] + in_S1 * dpre[16 * NT + k];
    double d157[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d157[k] = dpre[11 * NT + k] * t148 + pre[11] * d148[k];
    double d158[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d158[k] = d156[k] - d157[k];
    double d159[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d159[k] = d58[k] * pre[9] + t58 * dpre[9 * NT + k];
    double d160[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d160[k] = d158[k] - d159[k];
    double d161[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d161[k] = -d160[k];
    double d162[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d162[k] = din[5 * NT + k] * pre[16] + in_S2 * dpre[16 * NT + k];
    double d163[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d163[k] = dpre[12 * NT + k] * t148 + pre[12] * d148[k];
    double d164[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d164[k] = d162[k] - d163[k];
    double d165[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d165[k] = d61[k] * pre[9] + t61 * dpre[9 * NT + k];
    double d166[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d166[k] = d164[k] - d165[k];
    double d167[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d167[k] = -d166[k];
    double d168[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d168[k] = din[6 * NT + k] * pre[17] + in_H0 * dpre[17 * NT + k];
    double d169[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d169[k] = dpre[10 * NT + k] * t149 + pre[10] * d149[k];
    double d170[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d170[k] = d168[k] - d169[k];
    double d171[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d171[k] = d55[k] * pre[8] + t55 * dpre[8 * NT + k];
    double d172[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d172[k] = d170[k] - d171[k];
    double d173[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d173[k] = -d172[k];
    double d174[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d174[k] = din[7 * NT + k] * pre[17] + in_H1 * dpre[17 * NT + k];
    double d175[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d175[k] = dpre[11 * NT + k] * t149 + pre[11] * d149[k];
    double d176[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d176[k] = d174[k] - d175[k];
    double d177[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d177[k] = d58[k] * pre[8] + t58 * dpre[8 * NT + k];
    double d178[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d178[k] = d176[k] - d177[k];
    double d179[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d179[k] = -d178[k];
    double d180[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d180[k] = din[8 * NT + k] * pre[17] + in_H2 * dpre[17 * NT + k];
    double d181[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d181[k] = dpre[12 * NT + k] * t149 + pre[12] * d149[k];
    double d182[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d182[k] = d180[k] - d181[k];
    double d183[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d183[k] = d61[k] * pre[8] + t61 * dpre[8 * NT + k];
    double d184[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d184[k] = d182[k] - d183[k];
    double d185[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d185[k] = -d184[k];
    out[0] = t143;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[0 * NT + k] = d143[k];
    out[1] = t144;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[1 * NT + k] = d144[k];
    out[2] = t145;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[2 * NT + k] = d145[k];
    out[3] = t155;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[3 * NT + k] = d155[k];
    out[4] = t161;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[4 * NT + k] = d161[k];
    out[5] = t167;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[5 * NT + k] = d167[k];
    out[6] = t173;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[6 * NT + k] = d173[k];
    out[7] = t179;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[7 * NT + k] = d179[k];
    out[8] = t185;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[8 * NT + k] = d185[k];
}

// adj_flat: pre inputs (x, y, z); iteration inputs (hv0, hv1, hv2, S0, S1, S2, H0, H1, H2, P0, P1, P2, Q0, Q1, Q2);
// constants (R, hR, hk2f, hm, k2f, m)
constexpr int adj_flat_NPRE = 10;

// adj_flat: values fixed during a half kick (position, tidal parameters).
__host__ __device__ __forceinline__ void adj_flat_pre(double in_x, double in_y, double in_z,
        double c_R, double c_hR, double c_hk2f, double c_hm, double c_k2f, double c_m, double* __restrict__ pre) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t40 = c_m * c_hk2f;
    const double t41 = c_hR * c_hR;
    const double t42 = t41 * t41;
    const double t43 = c_hR * t42;
    const double t44 = t40 * t43;
    const double t46 = t44 * 0.16666666666666666;
    const double t47 = c_hm * c_k2f;
    const double t48 = c_R * c_R;
    const double t49 = t48 * t48;
    const double t50 = c_R * t49;
    const double t51 = t47 * t50;
    const double t52 = 0.16666666666666666 * t51;
    const double t53 = t23 * t23;
    const double t54 = t53 * t53;
    const double t55 = t23 * t54;
    const double t56 = t23 * t55;
    const double t57 = t23 * t56;
    const double t59 = 1.0 / t55;
    const double t61 = t46 * -6.0;
    const double t62 = t59 * t61;
    const double t64 = t52 * -6.0;
    const double t65 = t59 * t64;
    const double t78 = t59 * -3.0;
    const double t84 = 1.0 / t57;
    const double t85 = 15.0 * t84;
    const double t108 = 1.0 / c_m;
    pre[0] = in_x;
    pre[1] = in_y;
    pre[2] = in_z;
    pre[3] = t62;
    pre[4] = t65;
    pre[5] = t52;
    pre[6] = t46;
    pre[7] = t78;
    pre[8] = t85;
    pre[9] = t108;
}

// adj_flat: one midpoint iteration.  Outputs: a[3] (planet acceleration),
// dl[3] (planet dL/dt), th[3] (dL/dt of the host due to this planet).
__host__ __device__ __forceinline__ void adj_flat_iter(const double* __restrict__ pre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_R, double c_hR, double c_hk2f, double c_hm, double c_k2f, double c_m, double* __restrict__ out) {
    const double t30 = pre[0] * in_Q0;
    const double t31 = pre[1] * in_Q1;
    const double t32 = t30 + t31;
    const double t33 = pre[2] * in_Q2;
    const double t34 = t32 + t33;
    const double t35 = pre[0] * in_P0;
    const double t36 = pre[1] * in_P1;
    const double t37 = t35 + t36;
    const double t38 = pre[2] * in_P2;
    const double t39 = t37 + t38;
    const double t63 = t34 * pre[3];
    const double t66 = t39 * pre[4];
    const double t67 = in_S0 * in_S0;
    const double t68 = in_S1 * in_S1;
    const double t69 = t67 + t68;
    const double t70 = in_S2 * in_S2;
    const double t71 = t69 + t70;
    const double t72 = in_H0 * in_H0;
    const double t73 = in_H1 * in_H1;
    const double t74 = t72 + t73;
    const double t75 = in_H2 * in_H2;
    const double t76 = t74 + t75;
    const double t79 = pre[5] * t71;
    const double t80 = pre[6] * t76;
    const double t81 = t79 + t80;
    const double t82 = pre[7] * t81;
    const double t86 = t34 * pre[6];
    const double t87 = t34 * t86;
    const double t88 = t39 * pre[5];
    const double t89 = t39 * t88;
    const double t90 = t87 + t89;
    const double t91 = pre[8] * t90;
    const double t92 = t82 + t91;
    const double t93 = pre[0] * t92;
    const double t94 = in_S0 * t66;
    const double t95 = t93 + t94;
    const double t96 = in_H0 * t63;
    const double t97 = t95 + t96;
    const double t98 = pre[1] * t92;
    const double t99 = in_S1 * t66;
    const double t100 = t98 + t99;
    const double t101 = in_H1 * t63;
    const double t102 = t100 + t101;
    const double t103 = pre[2] * t92;
    const double t104 = in_S2 * t66;
    const double t105 = t103 + t104;
    const double t106 = in_H2 * t63;
    const double t107 = t105 + t106;
    const double t109 = t97 * pre[9];
    const double t110 = t102 * pre[9];
    const double t111 = t107 * pre[9];
    const double t112 = pre[1] * in_S2;
    const double t113 = pre[2] * in_S1;
    const double t114 = t112 - t113;
    const double t115 = pre[2] * in_S0;
    const double t116 = pre[0] * in_S2;
    const double t117 = t115 - t116;
    const double t118 = pre[0] * in_S1;
    const double t119 = pre[1] * in_S0;
    const double t120 = t118 - t119;
    const double t121 = pre[1] * in_H2;
    const double t122 = pre[2] * in_H1;
    const double t123 = t121 - t122;
    const double t124 = pre[2] * in_H0;
    const double t125 = pre[0] * in_H2;
    const double t126 = t124 - t125;
    const double t127 = pre[0] * in_H1;
    const double t128 = pre[1] * in_H0;
    const double t129 = t127 - t128;
    const double t130 = t66 * t114;
    const double t131 = -t130;
    const double t132 = t66 * t117;
    const double t133 = -t132;
    const double t134 = t66 * t120;
    const double t135 = -t134;
    const double t136 = t63 * t123;
    const double t137 = -t136;
    const double t138 = t63 * t126;
    const double t139 = -t138;
    const double t140 = t63 * t129;
    const double t141 = -t140;
    out[0] = t109;
    out[1] = t110;
    out[2] = t111;
    out[3] = t131;
    out[4] = t133;
    out[5] = t135;
    out[6] = t137;
    out[7] = t139;
    out[8] = t141;
}

// adj_flat: VJP of one iteration.  bin[15] += adjoints of (hv0, hv1, hv2, S0, S1, S2, H0, H1, H2, P0, P1, P2, Q0, Q1, Q2);
// bpre[adj_flat_NPRE] += adjoints of the pre values.
__host__ __device__ __forceinline__ void adj_flat_iter_vjp(const double* __restrict__ pre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_R, double c_hR, double c_hk2f, double c_hm, double c_k2f, double c_m, const double* __restrict__ bout, double* __restrict__ bin, double* __restrict__ bpre) {
    const double t30 = pre[0] * in_Q0;
    const double t31 = pre[1] * in_Q1;
    const double t32 = t30 + t31;
    const double t33 = pre[2] * in_Q2;
    const double t34 = t32 + t33;
    const double t35 = pre[0] * in_P0;
    const double t36 = pre[1] * in_P1;
    const double t37 = t35 + t36;
    const double t38 = pre[2] * in_P2;
    const double t39 = t37 + t38;
    const double t63 = t34 * pre[3];
    const double t66 = t39 * pre[4];
    const double t67 = in_S0 * in_S0;
    const double t68 = in_S1 * in_S1;
    const double t69 = t67 + t68;
    const double t70 = in_S2 * in_S2;
    const double t71 = t69 + t70;
    const double t72 = in_H0 * in_H0;
    const double t73 = in_H1 * in_H1;
    const double t74 = t72 + t73;
    const double t75 = in_H2 * in_H2;
    const double t76 = t74 + t75;
    const double t79 = pre[5] * t71;
    const double t80 = pre[6] * t76;
    const double t81 = t79 + t80;
    const double t82 = pre[7] * t81;
    const double t86 = t34 * pre[6];
    const double t87 = t34 * t86;
    const double t88 = t39 * pre[5];
    const double t89 = t39 * t88;
    const double t90 = t87 + t89;
    const double t91 = pre[8] * t90;
    const double t92 = t82 + t91;
    const double t93 = pre[0] * t92;
    const double t94 = in_S0 * t66;
    const double t95 = t93 + t94;
    const double t96 = in_H0 * t63;
    const double t97 = t95 + t96;
    const double t98 = pre[1] * t92;
    const double t99 = in_S1 * t66;
    const double t100 = t98 + t99;
    const double t101 = in_H1 * t63;
    const double t102 = t100 + t101;
    const double t103 = pre[2] * t92;
    const double t104 = in_S2 * t66;
    const double t105 = t103 + t104;
    const double t106 = in_H2 * t63;
    const double t107 = t105 + t106;
    const double t109 = t97 * pre[9];
    const double t110 = t102 * pre[9];
    const double t111 = t107 * pre[9];
    const double t112 = pre[1] * in_S2;
    const double t113 = pre[2] * in_S1;
    const double t114 = t112 - t113;
    const double t115 = pre[2] * in_S0;
    const double t116 = pre[0] * in_S2;
    const double t117 = t115 - t116;
    const double t118 = pre[0] * in_S1;
    const double t119 = pre[1] * in_S0;
    const double t120 = t118 - t119;
    const double t121 = pre[1] * in_H2;
    const double t122 = pre[2] * in_H1;
    const double t123 = t121 - t122;
    const double t124 = pre[2] * in_H0;
    const double t125 = pre[0] * in_H2;
    const double t126 = t124 - t125;
    const double t127 = pre[0] * in_H1;
    const double t128 = pre[1] * in_H0;
    const double t129 = t127 - t128;
    const double t130 = t66 * t114;
    const double t131 = -t130;
    const double t132 = t66 * t117;
    const double t133 = -t132;
    const double t134 = t66 * t120;
    const double t135 = -t134;
    const double t136 = t63 * t123;
    const double t137 = -t136;
    const double t138 = t63 * t126;
    const double t139 = -t138;
    const double t140 = t63 * t129;
    const double t141 = -t140;
    double b109 = bout[0];
    double b110 = bout[1];
    double b111 = bout[2];
    double b131 = bout[3];
    double b133 = bout[4];
    double b135 = bout[5];
    double b137 = bout[6];
    double b139 = bout[7];
    double b141 = bout[8];
    double b140 = -b141;
    double b63 = b140 * t129;
    double b129 = b140 * t63;
    double b138 = -b139;
    b63 += b138 * t126;
    double b126 = b138 * t63;
    double b136 = -b137;
    b63 += b136 * t123;
    double b123 = b136 * t63;
    double b134 = -b135;
    double b66 = b134 * t120;
    double b120 = b134 * t66;
    double b132 = -b133;
    b66 += b132 * t117;
    double b117 = b132 * t66;
    double b130 = -b131;
    b66 += b130 * t114;
    double b114 = b130 * t66;
    double b127 = b129;
    double b128 = -b129;
    bpre[1] += b128 * in_H0;
    double b_H0 = b128 * pre[1];
    bpre[0] += b127 * in_H1;
    double b_H1 = b127 * pre[0];
    double b124 = b126;
    double b125 = -b126;
    bpre[0] += b125 * in_H2;
    double b_H2 = b125 * pre[0];
    bpre[2] += b124 * in_H0;
    b_H0 += b124 * pre[2];
    double b121 = b123;
    double b122 = -b123;
    bpre[2] += b122 * in_H1;
    b_H1 += b122 * pre[2];
    bpre[1] += b121 * in_H2;
    b_H2 += b121 * pre[1];
    double b118 = b120;
    double b119 = -b120;
    bpre[1] += b119 * in_S0;
    double b_S0 = b119 * pre[1];
    bpre[0] += b118 * in_S1;
    double b_S1 = b118 * pre[0];
    double b115 = b117;
    double b116 = -b117;
    bpre[0] += b116 * in_S2;
    double b_S2 = b116 * pre[0];
    bpre[2] += b115 * in_S0;
    b_S0 += b115 * pre[2];
    double b112 = b114;
    double b113 = -b114;
    bpre[2] += b113 * in_S1;
    b_S1 += b113 * pre[2];
    bpre[1] += b112 * in_S2;
    b_S2 += b112 * pre[1];
    double b107 = b111 * pre[9];
    double b102 = b110 * pre[9];
    double b97 = b109 * pre[9];
    double b105 = b107;
    double b106 = b107;
    b_H2 += b106 * t63;
    b63 += b106 * in_H2;
    double b103 = b105;
    double b104 = b105;
    b_S2 += b104 * t66;
    b66 += b104 * in_S2;
    bpre[2] += b103 * t92;
    double b92 = b103 * pre[2];
    double b100 = b102;
    double b101 = b102;
    b_H1 += b101 * t63;
    b63 += b101 * in_H1;
    double b98 = b100;
    double b99 = b100;
    b_S1 += b99 * t66;
    b66 += b99 * in_S1;
    bpre[1] += b98 * t92;
    b92 += b98 * pre[1];
    double b95 = b97;
    double b96 = b97;
    b_H0 += b96 * t63;
    b63 += b96 * in_H0;
    double b93 = b95;
    double b94 = b95;
    b_S0 += b94 * t66;
    b66 += b94 * in_S0;
    bpre[0] += b93 * t92;
    b92 += b93 * pre[0];
    double b82 = b92;
    double b91 = b92;
    bpre[8] += b91 * t90;
    double b90 = b91 * pre[8];
    double b87 = b90;
    double b89 = b90;
    double b39 = b89 * t88;
    double b88 = b89 * t39;
    b39 += b88 * pre[5];
    double b34 = b87 * t86;
    double b86 = b87 * t34;
    b34 += b86 * pre[6];
    bpre[7] += b82 * t81;
    double b81 = b82 * pre[7];
    double b79 = b81;
    double b80 = b81;
    double b76 = b80 * pre[6];
    double b71 = b79 * pre[5];
    double b74 = b76;
    double b75 = b76;
    b_H2 += 2.0 * b75 * in_H2;
    double b72 = b74;
    double b73 = b74;
    b_H1 += 2.0 * b73 * in_H1;
    b_H0 += 2.0 * b72 * in_H0;
    double b69 = b71;
    double b70 = b71;
    b_S2 += 2.0 * b70 * in_S2;
    double b67 = b69;
    double b68 = b69;
    b_S1 += 2.0 * b68 * in_S1;
    b_S0 += 2.0 * b67 * in_S0;
    b39 += b66 * pre[4];
    bpre[4] += b66 * t39;
    b34 += b63 * pre[3];
    bpre[3] += b63 * t34;
    double b37 = b39;
    double b38 = b39;
    bpre[2] += b38 * in_P2;
    double b_P2 = b38 * pre[2];
    double b35 = b37;
    double b36 = b37;
    bpre[1] += b36 * in_P1;
    double b_P1 = b36 * pre[1];
    bpre[0] += b35 * in_P0;
    double b_P0 = b35 * pre[0];
    double b32 = b34;
    double b33 = b34;
    bpre[2] += b33 * in_Q2;
    double b_Q2 = b33 * pre[2];
    double b30 = b32;
    double b31 = b32;
    bpre[1] += b31 * in_Q1;
    double b_Q1 = b31 * pre[1];
    bpre[0] += b30 * in_Q0;
    double b_Q0 = b30 * pre[0];
    bin[3] += b_S0;
    bin[4] += b_S1;
    bin[5] += b_S2;
    bin[6] += b_H0;
    bin[7] += b_H1;
    bin[8] += b_H2;
    bin[9] += b_P0;
    bin[10] += b_P1;
    bin[11] += b_P2;
    bin[12] += b_Q0;
    bin[13] += b_Q1;
    bin[14] += b_Q2;
}

// adj_flat: VJP of the pre values.  bin[3] += adjoints of (x, y, z).
__host__ __device__ __forceinline__ void adj_flat_pre_vjp(double in_x, double in_y, double in_z,
        double c_R, double c_hR, double c_hk2f, double c_hm, double c_k2f, double c_m, const double* __restrict__ bpre, double* __restrict__ bin) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t40 = c_m * c_hk2f;
    const double t41 = c_hR * c_hR;
    const double t42 = t41 * t41;
    const double t43 = c_hR * t42;
    const double t44 = t40 * t43;
    const double t46 = t44 * 0.16666666666666666;
    const double t47 = c_hm * c_k2f;
    const double t48 = c_R * c_R;
    const double t49 = t48 * t48;
    const double t50 = c_R * t49;
    const double t51 = t47 * t50;
    const double t52 = 0.16666666666666666 * t51;
    const double t53 = t23 * t23;
    const double t54 = t53 * t53;
    const double t55 = t23 * t54;
    const double t56 = t23 * t55;
    const double t57 = t23 * t56;
    const double t59 = 1.0 / t55;
    const double t61 = t46 * -6.0;
    const double t62 = t59 * t61;
    const double t64 = t52 * -6.0;
    const double t65 = t59 * t64;
    const double t78 = t59 * -3.0;
    const double t84 = 1.0 / t57;
    const double t85 = 15.0 * t84;
    const double t108 = 1.0 / c_m;
    double b_x = bpre[0];
    double b_y = bpre[1];
    double b_z = bpre[2];
    double b62 = bpre[3];
    double b65 = bpre[4];
    double b78 = bpre[7];
    double b85 = bpre[8];
    double b84 = b85 * 15.0;
    double b57 = -b84 * t84 * t84;
    double b59 = b78 * -3.0;
    b59 += b65 * t64;
    b59 += b62 * t61;
    double b55 = -b59 * t59 * t59;
    double b23 = b57 * t56;
    double b56 = b57 * t23;
    b23 += b56 * t55;
    b55 += b56 * t23;
    b23 += b55 * t54;
    double b54 = b55 * t23;
    double b53 = 2.0 * b54 * t53;
    b23 += 2.0 * b53 * t23;
    double b22 = 0.5 * b23 / t23;
    double b20 = b22;
    double b21 = b22;
    b_z += 2.0 * b21 * in_z;
    double b18 = b20;
    double b19 = b20;
    b_y += 2.0 * b19 * in_y;
    b_x += 2.0 * b18 * in_x;
    bin[0] += b_x;
    bin[1] += b_y;
    bin[2] += b_z;
}

// adj_flat: pre values and their tangents (din[i * NT + k]: tangent k of pre input i).
template <int NT>
__host__ __device__ __forceinline__ void adj_flat_pre_jvp(double in_x, double in_y, double in_z,
        double c_R, double c_hR, double c_hk2f, double c_hm, double c_k2f, double c_m, const double* __restrict__ din, double* __restrict__ pre,
        double* __restrict__ dpre) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t40 = c_m * c_hk2f;
    const double t41 = c_hR * c_hR;
    const double t42 = t41 * t41;
    const double t43 = c_hR * t42;
    const double t44 = t40 * t43;
    const double t46 = t44 * 0.16666666666666666;
    const double t47 = c_hm * c_k2f;
    const double t48 = c_R * c_R;
    const double t49 = t48 * t48;
    const double t50 = c_R * t49;
    const double t51 = t47 * t50;
    const double t52 = 0.16666666666666666 * t51;
    const double t53 = t23 * t23;
    const double t54 = t53 * t53;
    const double t55 = t23 * t54;
    const double t56 = t23 * t55;
    const double t57 = t23 * t56;
    const double t59 = 1.0 / t55;
    const double t61 = t46 * -6.0;
    const double t62 = t59 * t61;
    const double t64 = t52 * -6.0;
    const double t65 = t59 * t64;
    const double t78 = t59 * -3.0;
    const double t84 = 1.0 / t57;
    const double t85 = 15.0 * t84;
    const double t108 = 1.0 / c_m;
    double d18[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d18[k] = 2.0 * in_x * din[0 * NT + k];
    double d19[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d19[k] = 2.0 * in_y * din[1 * NT + k];
    double d20[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d20[k] = d18[k] + d19[k];
    double d21[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d21[k] = 2.0 * in_z * din[2 * NT + k];
    double d22[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d22[k] = d20[k] + d21[k];
    double d23[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d23[k] = 0.5 * d22[k] / t23;
    double d53[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d53[k] = 2.0 * t23 * d23[k];
    double d54[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d54[k] = 2.0 * t53 * d53[k];
    double d55[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d55[k] = d23[k] * t54 + t23 * d54[k];
    double d56[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d56[k] = d23[k] * t55 + t23 * d55[k];
    double d57[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d57[k] = d23[k] * t56 + t23 * d56[k];
    double d59[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d59[k] = -t59 * t59 * d55[k];
    double d62[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d62[k] = d59[k] * t61;
    double d65[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d65[k] = d59[k] * t64;
    double d78[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d78[k] = d59[k] * -3.0;
    double d84[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d84[k] = -t84 * t84 * d57[k];
    double d85[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d85[k] = 15.0 * d84[k];
    pre[0] = in_x;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[0 * NT + k] = din[0 * NT + k];
    pre[1] = in_y;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[1 * NT + k] = din[1 * NT + k];
    pre[2] = in_z;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[2 * NT + k] = din[2 * NT + k];
    pre[3] = t62;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[3 * NT + k] = d62[k];
    pre[4] = t65;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[4 * NT + k] = d65[k];
    pre[5] = t52;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[5 * NT + k] = 0.0;
    pre[6] = t46;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[6 * NT + k] = 0.0;
    pre[7] = t78;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[7 * NT + k] = d78[k];
    pre[8] = t85;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[8 * NT + k] = d85[k];
    pre[9] = t108;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[9 * NT + k] = 0.0;
}

// adj_flat: one iteration, outputs and their tangents (din[i * NT + k] for the
// iteration inputs; dout[o * NT + k]).
template <int NT>
__host__ __device__ __forceinline__ void adj_flat_iter_jvp(const double* __restrict__ pre,
        const double* __restrict__ dpre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_R, double c_hR, double c_hk2f, double c_hm, double c_k2f, double c_m, const double* __restrict__ din, double* __restrict__ out,
        double* __restrict__ dout) {
    const double t30 = pre[0] * in_Q0;
    const double t31 = pre[1] * in_Q1;
    const double t32 = t30 + t31;
    const double t33 = pre[2] * in_Q2;
    const double t34 = t32 + t33;
    const double t35 = pre[0] * in_P0;
    const double t36 = pre[1] * in_P1;
    const double t37 = t35 + t36;
    const double t38 = pre[2] * in_P2;
    const double t39 = t37 + t38;
    const double t63 = t34 * pre[3];
    const double t66 = t39 * pre[4];
    const double t67 = in_S0 * in_S0;
    const double t68 = in_S1 * in_S1;
    const double t69 = t67 + t68;
    const double t70 = in_S2 * in_S2;
    const double t71 = t69 + t70;
    const double t72 = in_H0 * in_H0;
    const double t73 = in_H1 * in_H1;
    const double t74 = t72 + t73;
    const double t75 = in_H2 * in_H2;
    const double t76 = t74 + t75;
    const double t79 = pre[5] * t71;
    const double t80 = pre[6] * t76;
    const double t81 = t79 + t80;
    const double t82 = pre[7] * t81;
    const double t86 = t34 * pre[6];
    const double t87 = t34 * t86;
    const double t88 = t39 * pre[5];
    const double t89 = t39 * t88;
    const double t90 = t87 + t89;
    const double t91 = pre[8] * t90;
    const double t92 = t82 + t91;
    const double t93 = pre[0] * t92;
    const double t94 = in_S0 * t66;
    const double t95 = t93 + t94;
    const double t96 = in_H0 * t63;
    const double t97 = t95 + t96;
    const double t98 = pre[1] * t92;
    const double t99 = in_S1 * t66;
    const double t100 = t98 + t99;
    const double t101 = in_H1 * t63;
    const double t102 = t100 + t101;
    const double t103 = pre[2] * t92;
    const double t104 = in_S2 * t66;
    const double t105 = t103 + t104;
    const double t106 = in_H2 * t63;
    const double t107 = t105 + t106;
    const double t109 = t97 * pre[9];
    const double t110 = t102 * pre[9];
    const double t111 = t107 * pre[9];
    const double t112 = pre[1] * in_S2;
    const double t113 = pre[2] * in_S1;
    const double t114 = t112 - t113;
    const double t115 = pre[2] * in_S0;
    const double t116 = pre[0] * in_S2;
    const double t117 = t115 - t116;
    const double t118 = pre[0] * in_S1;
    const double t119 = pre[1] * in_S0;
    const double t120 = t118 - t119;
    const double t121 = pre[1] * in_H2;
    const double t122 = pre[2] * in_H1;
    const double t123 = t121 - t122;
    const double t124 = pre[2] * in_H0;
    const double t125 = pre[0] * in_H2;
    const double t126 = t124 - t125;
    const double t127 = pre[0] * in_H1;
    const double t128 = pre[1] * in_H0;
    const double t129 = t127 - t128;
    const double t130 = t66 * t114;
    const double t131 = -t130;
    const double t132 = t66 * t117;
    const double t133 = -t132;
    const double t134 = t66 * t120;
    const double t135 = -t134;
    const double t136 = t63 * t123;
    const double t137 = -t136;
    const double t138 = t63 * t126;
    const double t139 = -t138;
    const double t140 = t63 * t129;
    const double t141 = -t140;
    double d30[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d30[k] = dpre[0 * NT + k] * in_Q0 + pre[0] * din[12 * NT + k];
    double d31[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d31[k] = dpre[1 * NT + k] * in_Q1 + pre[1] * din[13 * NT + k];
    double d32[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d32[k] = d30[k] + d31[k];
    double d33[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d33[k] = dpre[2 * NT + k] * in_Q2 + pre[2] * din[14 * NT + k];
    double d34[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d34[k] = d32[k] + d33[k];
    double d35[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d35[k] = dpre[0 * NT + k] * in_P0 + pre[0] * din[9 * NT + k];
    double d36[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d36[k] = dpre[1 * NT + k] * in_P1 + pre[1] * din[10 * NT + k];
    double d37[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d37[k] = d35[k] + d36[k];
    double d38[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d38[k] = dpre[2 * NT + k] * in_P2 + pre[2] * din[11 * NT + k];
    double d39[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d39[k] = d37[k] + d38[k];
    double d63[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d63[k] = d34[k] * pre[3] + t34 * dpre[3 * NT + k];
    double d66[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d66[k] = d39[k] * pre[4] + t39 * dpre[4 * NT + k];
    double d67[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d67[k] = 2.0 * in_S0 * din[3 * NT + k];
    double d68[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d68[k] = 2.0 * in_S1 * din[4 * NT + k];
    double d69[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d69[k] = d67[k] + d68[k];
    double d70[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d70[k] = 2.0 * in_S2 * din[5 * NT + k];
    double d71[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d71[k] = d69[k] + d70[k];
    double d72[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d72[k] = 2.0 * in_H0 * din[6 * NT + k];
    double d73[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d73[k] = 2.0 * in_H1 * din[7 * NT + k];
    double d74[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d74[k] = d72[k] + d73[k];
    double d75[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d75[k] = 2.0 * in_H2 * din[8 * NT + k];
    double d76[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d76[k] = d74[k] + d75[k];
    double d79[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d79[k] = pre[5] * d71[k];
    double d80[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d80[k] = pre[6] * d76[k];
    double d81[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d81[k] = d79[k] + d80[k];
    double d82[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d82[k] = dpre[7 * NT + k] * t81 + pre[7] * d81[k];
    double d86[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d86[k] = d34[k] * pre[6];
    double d87[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d87[k] = d34[k] * t86 + t34 * d86[k];
    double d88[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d88[k] = d39[k] * pre[5];
    double d89[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d89[k] = d39[k] * t88 + t39 * d88[k];
    double d90[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d90[k] = d87[k] + d89[k];
    double d91[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d91[k] = dpre[8 * NT + k] * t90 + pre[8] * d90[k];
    double d92[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d92[k] = d82[k] + d91[k];
    double d93[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d93[k] = dpre[0 * NT + k] * t92 + pre[0] * d92[k];
    double d94[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d94[k] = din[3 * NT + k] * t66 + in_S0 * d66[k];
    double d95[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d95[k] = d93[k] + d94[k];
    double d96[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d96[k] = din[6 * NT + k] * t63 + in_H0 * d63[k];
    double d97[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d97[k] = d95[k] + d96[k];
    double d98[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d98[k] = dpre[1 * NT + k] * t92 + pre[1] * d92[k];
    double d99[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d99[k] = din[4 * NT + k] * t66 + in_S1 * d66[k];
    double d100[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d100[k] = d98[k] + d99[k];
    double d101[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d101[k] = din[7 * NT + k] * t63 + in_H1 * d63[k];
    double d102[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d102[k] = d100[k] + d101[k];
    double d103[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d103[k] = dpre[2 * NT + k] * t92 + pre[2] * d92[k];
    double d104[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d104[k] = din[5 * NT + k] * t66 + in_S2 * d66[k];
    double d105[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d105[k] = d103[k] + d104[k];
    double d106[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d106[k] = din[8 * NT + k] * t63 + in_H2 * d63[k];
    double d107[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d107[k] = d105[k] + d106[k];
    double d109[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d109[k] = d97[k] * pre[9];
    double d110[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d110[k] = d102[k] * pre[9];
    double d111[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d111[k] = d107[k] * pre[9];
    double d112[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d112[k] = dpre[1 * NT + k] * in_S2 + pre[1] * din[5 * NT + k];
    double d113[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d113[k] = dpre[2 * NT + k] * in_S1 + pre[2] * din[4 * NT + k];
    double d114[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d114[k] = d112[k] - d113[k];
    double d115[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d115[k] = dpre[2 * NT + k] * in_S0 + pre[2] * din[3 * NT + k];
    double d116[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d116[k] = dpre[0 * NT + k] * in_S2 + pre[0] * din[5 * NT + k];
    double d117[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d117[k] = d115[k] - d116[k];
    double d118[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d118[k] = dpre[0 * NT + k] * in_S1 + pre[0] * din[4 * NT + k];
    double d119[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d119[k] = dpre[1 * NT + k] * in_S0 + pre[1] * din[3 * NT + k];
    double d120[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d120[k] = d118[k] - d119[k];
    double d121[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d121[k] = dpre[1 * NT + k] * in_H2 + pre[1] * din[8 * NT + k];
    double d122[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d122[k] = dpre[2 * NT + k] * in_H1 + pre[2] * din[7 * NT + k];
    double d123[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d123[k] = d121[k] - d122[k];
    double d124[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d124[k] = dpre[2 * NT + k] * in_H0 + pre[2] * din[6 * NT + k];
    double d125[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d125[k] = dpre[0 * NT + k] * in_H2 + pre[0] * din[8 * NT + k];
    double d126[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d126[k] = d124[k] - d125[k];
    double d127[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d127[k] = dpre[0 * NT + k] * in_H1 + pre[0] * din[7 * NT + k];
    double d128[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d128[k] = dpre[1 * NT + k] * in_H0 + pre[1] * din[6 * NT + k];
    double d129[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d129[k] = d127[k] - d128[k];
    double d130[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d130[k] = d66[k] * t114 + t66 * d114[k];
    double d131[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d131[k] = -d130[k];
    double d132[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d132[k] = d66[k] * t117 + t66 * d117[k];
    double d133[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d133[k] = -d132[k];
    double d134[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d134[k] = d66[k] * t120 + t66 * d120[k];
    double d135[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d135[k] = -d134[k];
    double d136[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d136[k] = d63[k] * t123 + t63 * d123[k];
    double d137[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d137[k] = -d136[k];
    double d138[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d138[k] = d63[k] * t126 + t63 * d126[k];
    double d139[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d139[k] = -d138[k];
    double d140[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d140[k] = d63[k] * t129 + t63 * d129[k];
    double d141[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d141[k] = -d140[k];
    out[0] = t109;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[0 * NT + k] = d109[k];
    out[1] = t110;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[1 * NT + k] = d110[k];
    out[2] = t111;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[2 * NT + k] = d111[k];
    out[3] = t131;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[3 * NT + k] = d131[k];
    out[4] = t133;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[4 * NT + k] = d133[k];
    out[5] = t135;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[5 * NT + k] = d135[k];
    out[6] = t137;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[6 * NT + k] = d137[k];
    out[7] = t139;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[7 * NT + k] = d139[k];
    out[8] = t141;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[8 * NT + k] = d141[k];
}

// adj_gr: pre inputs (x, y, z); iteration inputs (hv0, hv1, hv2, S0, S1, S2, H0, H1, H2, P0, P1, P2, Q0, Q1, Q2);
// constants (hm, hmg, hmoi, m, mg, moi)
constexpr int adj_gr_NPRE = 24;

// adj_gr: values fixed during a half kick (position, tidal parameters).
__host__ __device__ __forceinline__ void adj_gr_pre(double in_x, double in_y, double in_z,
        double c_hm, double c_hmg, double c_hmoi, double c_m, double c_mg, double c_moi, double* __restrict__ pre) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t33 = 1.0 / t23;
    const double t34 = in_x * t33;
    const double t35 = in_y * t33;
    const double t36 = in_z * t33;
    const double t48 = c_mg + c_hmg;
    const double t49 = c_mg * c_hmg;
    const double t50 = t48 * t48;
    const double t51 = 1.0 / t50;
    const double t52 = t49 * t51;
    const double t53 = t23 * t23;
    const double t54 = t33 * t48;
    const double t55 = -t48;
    const double t56 = kC2 * t53;
    const double t57 = 1.0 / t56;
    const double t58 = t55 * t57;
    const double t60 = t52 * 3.0;
    const double t61 = 1.0 + t60;
    const double t63 = t52 + 2.0;
    const double t64 = 2.0 * t63;
    const double t65 = t54 * t64;
    const double t67 = t52 * 1.5;
    const double t68 = t48 * t57;
    const double t69 = 2.0 * t68;
    const double t70 = 2.0 - t52;
    const double t71 = t69 * t70;
    const double t73 = t52 * 29.0;
    const double t75 = t73 + 12.0;
    const double t77 = t75 * 0.75;
    const double t78 = 1.0 / t53;
    const double t79 = t50 * t78;
    const double t80 = t77 * t79;
    const double t82 = t52 * 4.0;
    const double t83 = 3.0 - t82;
    const double t84 = t52 * t83;
    const double t86 = t52 * 1.875;
    const double t87 = 1.0 - t60;
    const double t88 = t86 * t87;
    const double t89 = t67 * t83;
    const double t91 = t52 * 0.5;
    const double t93 = 13.0 - t82;
    const double t94 = t91 * t93;
    const double t95 = t54 * t94;
    const double t97 = t52 * 25.0;
    const double t98 = 2.0 + t97;
    const double t99 = t52 * 2.0;
    const double t100 = t52 * t99;
    const double t101 = t98 + t100;
    const double t102 = t54 * t101;
    const double t104 = t58 * -0.5;
    const double t106 = t82 + 15.0;
    const double t107 = t52 * t106;
    const double t109 = t52 * 41.0;
    const double t110 = 4.0 + t109;
    const double t112 = t52 * 8.0;
    const double t113 = t52 * t112;
    const double t114 = t110 + t113;
    const double t115 = t54 * t114;
    const double t116 = 3.0 + t99;
    const double t117 = t60 * t116;
    const double t118 = t80 - t65;
    const double t119 = t61 - t95;
    const double t120 = t67 + t102;
    const double t121 = -t120;
    const double t122 = t104 * t115;
    const double t123 = t71 - t122;
    const double t124 = t104 * t107;
    const double t125 = t104 * t117;
    const double t126 = -t125;
    const double t159 = c_hm - c_m;
    const double t160 = c_moi * t159;
    const double t161 = 1.0 / c_m;
    const double t162 = t160 * t161;
    const double t163 = 1.0 / c_hm;
    const double t164 = t159 * t163;
    const double t187 = t34 * 6.0;
    const double t188 = t33 * t187;
    const double t189 = t35 * 6.0;
    const double t190 = t33 * t189;
    const double t191 = t36 * 6.0;
    const double t192 = t33 * t191;
    const double t255 = c_m * c_hm;
    const double t256 = c_m + c_hm;
    const double t257 = 1.0 / t256;
    const double t258 = t255 * t257;
    const double t259 = c_m * 1.5;
    const double t260 = t163 * t259;
    const double t261 = 2.0 + t260;
    const double t262 = t258 * t261;
    const double t263 = c_hm * 1.5;
    const double t264 = t161 * t263;
    const double t265 = 2.0 + t264;
    const double t266 = t258 * t265;
    pre[0] = in_x;
    pre[1] = in_y;
    pre[2] = in_z;
    pre[3] = t33;
    pre[4] = t84;
    pre[5] = t119;
    pre[6] = t89;
    pre[7] = t118;
    pre[8] = t88;
    pre[9] = t121;
    pre[10] = t58;
    pre[11] = t124;
    pre[12] = t123;
    pre[13] = t126;
    pre[14] = t34;
    pre[15] = t35;
    pre[16] = t36;
    pre[17] = t162;
    pre[18] = t164;
    pre[19] = t188;
    pre[20] = t190;
    pre[21] = t192;
    pre[22] = t262;
    pre[23] = t266;
}

// adj_gr: one midpoint iteration.  Outputs: a[3] (planet acceleration),
// dl[3] (planet dL/dt), th[3] (dL/dt of the host due to this planet).
__host__ __device__ __forceinline__ void adj_gr_iter(const double* __restrict__ pre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_hm, double c_hmg, double c_hmoi, double c_m, double c_mg, double c_moi, double* __restrict__ out) {
    const double t37 = pre[0] * in_hv0;
    const double t38 = pre[1] * in_hv1;
    const double t39 = t37 + t38;
    const double t40 = pre[2] * in_hv2;
    const double t41 = t39 + t40;
    const double t42 = pre[3] * t41;
    const double t43 = in_hv0 * in_hv0;
    const double t44 = in_hv1 * in_hv1;
    const double t45 = t43 + t44;
    const double t46 = in_hv2 * in_hv2;
    const double t47 = t45 + t46;
    const double t127 = t42 * t42;
    const double t128 = t47 * pre[4];
    const double t129 = pre[5] + t128;
    const double t130 = pre[6] * t127;
    const double t131 = t129 - t130;
    const double t132 = t47 * t131;
    const double t133 = pre[7] + t132;
    const double t134 = pre[8] * t127;
    const double t135 = pre[9] + t134;
    const double t136 = t127 * t135;
    const double t137 = t133 + t136;
    const double t138 = pre[10] * t137;
    const double t139 = t47 * pre[11];
    const double t140 = pre[12] + t139;
    const double t141 = pre[13] * t127;
    const double t142 = t140 + t141;
    const double t143 = t42 * t142;
    const double t144 = pre[14] * t138;
    const double t145 = in_hv0 * t143;
    const double t146 = t144 + t145;
    const double t147 = pre[15] * t138;
    const double t148 = in_hv1 * t143;
    const double t149 = t147 + t148;
    const double t150 = pre[16] * t138;
    const double t151 = in_hv2 * t143;
    const double t152 = t150 + t151;
    const double t153 = in_H0 * c_hmoi;
    const double t154 = in_H1 * c_hmoi;
    const double t155 = in_H2 * c_hmoi;
    const double t156 = in_S0 * c_moi;
    const double t157 = in_S1 * c_moi;
    const double t158 = in_S2 * c_moi;
    const double t165 = in_S0 * pre[17];
    const double t166 = t153 * pre[18];
    const double t167 = t165 - t166;
    const double t168 = in_S1 * pre[17];
    const double t169 = t154 * pre[18];
    const double t170 = t168 - t169;
    const double t171 = in_S2 * pre[17];
    const double t172 = t155 * pre[18];
    const double t173 = t171 - t172;
    const double t174 = t153 + t156;
    const double t175 = t154 + t157;
    const double t176 = t155 + t158;
    const double t177 = pre[1] * in_hv2;
    const double t178 = pre[2] * in_hv1;
    const double t179 = t177 - t178;
    const double t180 = pre[2] * in_hv0;
    const double t181 = pre[0] * in_hv2;
    const double t182 = t180 - t181;
    const double t183 = pre[0] * in_hv1;
    const double t184 = pre[1] * in_hv0;
    const double t185 = t183 - t184;
    const double t193 = 2.0 * t174;
    const double t194 = t167 + t193;
    const double t195 = t179 * t194;
    const double t196 = pre[19] * t195;
    const double t197 = 2.0 * t175;
    const double t198 = t170 + t197;
    const double t199 = t182 * t198;
    const double t200 = pre[20] * t199;
    const double t201 = 2.0 * t176;
    const double t202 = t173 + t201;
    const double t203 = t185 * t202;
    const double t204 = pre[21] * t203;
    const double t205 = pre[14] * t42;
    const double t206 = t205 - in_hv0;
    const double t207 = pre[15] * t42;
    const double t208 = t207 - in_hv1;
    const double t209 = pre[16] * t42;
    const double t210 = t209 - in_hv2;
    const double t211 = t42 * 2.0;
    const double t213 = t206 * 7.0;
    const double t214 = pre[14] * t211;
    const double t215 = t213 + t214;
    const double t216 = t208 * 7.0;
    const double t217 = pre[15] * t211;
    const double t218 = t216 + t217;
    const double t219 = t210 * 7.0;
    const double t220 = pre[16] * t211;
    const double t221 = t219 + t220;
    const double t222 = t176 * t218;
    const double t223 = t175 * t221;
    const double t224 = t222 - t223;
    const double t225 = t174 * t221;
    const double t226 = t176 * t215;
    const double t227 = t225 - t226;
    const double t228 = t175 * t215;
    const double t229 = t174 * t218;
    const double t230 = t228 - t229;
    const double t231 = t173 * t208;
    const double t232 = t170 * t210;
    const double t233 = t231 - t232;
    const double t234 = t167 * t210;
    const double t235 = t173 * t206;
    const double t236 = t234 - t235;
    const double t237 = t170 * t206;
    const double t238 = t167 * t208;
    const double t239 = t237 - t238;
    const double t240 = t196 + t224;
    const double t241 = 3.0 * t233;
    const double t242 = t240 + t241;
    const double t243 = kFA * t242;
    const double t244 = t146 + t243;
    const double t245 = t200 + t227;
    const double t246 = 3.0 * t236;
    const double t247 = t245 + t246;
    const double t248 = kFA * t247;
    const double t249 = t149 + t248;
    const double t250 = t204 + t230;
    const double t251 = 3.0 * t239;
    const double t252 = t250 + t251;
    const double t253 = kFA * t252;
    const double t254 = t152 + t253;
    const double t267 = pre[14] * t156;
    const double t268 = pre[15] * t157;
    const double t269 = t267 + t268;
    const double t270 = pre[16] * t158;
    const double t271 = t269 + t270;
    const double t272 = 3.0 * t271;
    const double t273 = pre[14] * t153;
    const double t274 = pre[15] * t154;
    const double t275 = t273 + t274;
    const double t276 = pre[16] * t155;
    const double t277 = t275 + t276;
    const double t278 = 3.0 * t277;
    const double t279 = t179 * pre[22];
    const double t280 = t279 - t156;
    const double t281 = pre[14] * t272;
    const double t282 = t280 + t281;
    const double t283 = t182 * pre[22];
    const double t284 = t283 - t157;
    const double t285 = pre[15] * t272;
    const double t286 = t284 + t285;
    const double t287 = t185 * pre[22];
    const double t288 = t287 - t158;
    const double t289 = pre[16] * t272;
    const double t290 = t288 + t289;
    const double t291 = t179 * pre[23];
    const double t292 = t291 - t153;
    const double t293 = pre[14] * t278;
    const double t294 = t292 + t293;
    const double t295 = t182 * pre[23];
    const double t296 = t295 - t154;
    const double t297 = pre[15] * t278;
    const double t298 = t296 + t297;
    const double t299 = t185 * pre[23];
    const double t300 = t299 - t155;
    const double t301 = pre[16] * t278;
    const double t302 = t300 + t301;
    const double t303 = t155 * t286;
    const double t304 = t154 * t290;
    const double t305 = t303 - t304;
    const double t306 = t153 * t290;
    const double t307 = t155 * t282;
    const double t308 = t306 - t307;
    const double t309 = t154 * t282;
    const double t310 = t153 * t286;
    const double t311 = t309 - t310;
    const double t312 = t158 * t298;
    const double t313 = t157 * t302;
    const double t314 = t312 - t313;
    const double t315 = t156 * t302;
    const double t316 = t158 * t294;
    const double t317 = t315 - t316;
    const double t318 = t157 * t294;
    const double t319 = t156 * t298;
    const double t320 = t318 - t319;
    const double t321 = kFA * t305;
    const double t322 = kFA * t308;
    const double t323 = kFA * t311;
    const double t324 = kFA * t314;
    const double t325 = kFA * t317;
    const double t326 = kFA * t320;
    out[0] = t244;
    out[1] = t249;
    out[2] = t254;
    out[3] = t324;
    out[4] = t325;
    out[5] = t326;
    out[6] = t321;
    out[7] = t322;
    out[8] = t323;
}

// adj_gr: VJP of one iteration.  bin[15] += adjoints of (hv0, hv1, hv2, S0, S1, S2, H0, H1, H2, P0, P1, P2, Q0, Q1, Q2);
// bpre[adj_gr_NPRE] += adjoints of the pre values.
__host__ __device__ __forceinline__ void adj_gr_iter_vjp(const double* __restrict__ pre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_hm, double c_hmg, double c_hmoi, double c_m, double c_mg, double c_moi, const double* __restrict__ bout, double* __restrict__ bin, double* __restrict__ bpre) {
    const double t37 = pre[0] * in_hv0;
    const double t38 = pre[1] * in_hv1;
    const double t39 = t37 + t38;
    const double t40 = pre[2] * in_hv2;
    const double t41 = t39 + t40;
    const double t42 = pre[3] * t41;
    const double t43 = in_hv0 * in_hv0;
    const double t44 = in_hv1 * in_hv1;
    const double t45 = t43 + t44;
    const double t46 = in_hv2 * in_hv2;
    const double t47 = t45 + t46;
    const double t127 = t42 * t42;
    const double t128 = t47 * pre[4];
    const double t129 = pre[5] + t128;
    const double t130 = pre[6] * t127;
    const double t131 = t129 - t130;
    const double t132 = t47 * t131;
    const double t133 = pre[7] + t132;
    const double t134 = pre[8] * t127;
    const double t135 = pre[9] + t134;
    const double t136 = t127 * t135;
    const double t137 = t133 + t136;
    const double t138 = pre[10] * t137;
    const double t139 = t47 * pre[11];
    const double t140 = pre[12] + t139;
    const double t141 = pre[13] * t127;
    const double t142 = t140 + t141;
    const double t143 = t42 * t142;
    const double t144 = pre[14] * t138;
    const double t145 = in_hv0 * t143;
    const double t146 = t144 + t145;
    const double t147 = pre[15] * t138;
    const double t148 = in_hv1 * t143;
    const double t149 = t147 + t148;
    const double t150 = pre[16] * t138;
    const double t151 = in_hv2 * t143;
    const double t152 = t150 + t151;
    const double t153 = in_H0 * c_hmoi;
    const double t154 = in_H1 * c_hmoi;
    const double t155 = in_H2 * c_hmoi;
    const double t156 = in_S0 * c_moi;
    const double t157 = in_S1 * c_moi;
    const double t158 = in_S2 * c_moi;
    const double t165 = in_S0 * pre[17];
    const double t166 = t153 * pre[18];
    const double t167 = t165 - t166;
    const double t168 = in_S1 * pre[17];
    const double t169 = t154 * pre[18];
    const double t170 = t168 - t169;
    const double t171 = in_S2 * pre[17];
    const double t172 = t155 * pre[18];
    const double t173 = t171 - t172;
    const double t174 = t153 + t156;
    const double t175 = t154 + t157;
    const double t176 = t155 + t158;
    const double t177 = pre[1] * in_hv2;
    const double t178 = pre[2] * in_hv1;
    const double t179 = t177 - t178;
    const double t180 = pre[2] * in_hv0;
    const double t181 = pre[0] * in_hv2;
    const double t182 = t180 - t181;
    const double t183 = pre[0] * in_hv1;
    const double t184 = pre[1] * in_hv0;
    const double t185 = t183 - t184;
    const double t193 = 2.0 * t174;
    const double t194 = t167 + t193;
    const double t195 = t179 * t194;
    const double t196 = pre[19] * t195;
    const double t197 = 2.0 * t175;
    const double t198 = t170 + t197;
    const double t199 = t182 * t198;
    const double t200 = pre[20] * t199;
    const double t201 = 2.0 * t176;
    const double t202 = t173 + t201;
    const double t203 = t185 * t202;
    const double t204 = pre[21] * t203;
    const double t205 = pre[14] * t42;
    const double t206 = t205 - in_hv0;
    const double t207 = pre[15] * t42;
    const double t208 = t207 - in_hv1;
    const double t209 = pre[16] * t42;
    const double t210 = t209 - in_hv2;
    const double t211 = t42 * 2.0;
    const double t213 = t206 * 7.0;
    const double t214 = pre[14] * t211;
    const double t215 = t213 + t214;
    const double t216 = t208 * 7.0;
    const double t217 = pre[15] * t211;
    const double t218 = t216 + t217;
    const double t219 = t210 * 7.0;
    const double t220 = pre[16] * t211;
    const double t221 = t219 + t220;
    const double t222 = t176 * t218;
    const double t223 = t175 * t221;
    const double t224 = t222 - t223;
    const double t225 = t174 * t221;
    const double t226 = t176 * t215;
    const double t227 = t225 - t226;
    const double t228 = t175 * t215;
    const double t229 = t174 * t218;
    const double t230 = t228 - t229;
    const double t231 = t173 * t208;
    const double t232 = t170 * t210;
    const double t233 = t231 - t232;
    const double t234 = t167 * t210;
    const double t235 = t173 * t206;
    const double t236 = t234 - t235;
    const double t237 = t170 * t206;
    const double t238 = t167 * t208;
    const double t239 = t237 - t238;
    const double t240 = t196 + t224;
    const double t241 = 3.0 * t233;
    const double t242 = t240 + t241;
    const double t243 = kFA * t242;
    const double t244 = t146 + t243;
    const double t245 = t200 + t227;
    const double t246 = 3.0 * t236;
    const double t247 = t245 + t246;
    const double t248 = kFA * t247;
    const double t249 = t149 + t248;
    const double t250 = t204 + t230;
    const double t251 = 3.0 * t239;
    const double t252 = t250 + t251;
    const double t253 = kFA * t252;
    const double t254 = t152 + t253;
    const double t267 = pre[14] * t156;
    const double t268 = pre[15] * t157;
    const double t269 = t267 + t268;
    const double t270 = pre[16] * t158;
    const double t271 = t269 + t270;
    const double t272 = 3.0 * t271;
    const double t273 = pre[14] * t153;
    const double t274 = pre[15] * t154;
    const double t275 = t273 + t274;
    const double t276 = pre[16] * t155;
    const double t277 = t275 + t276;
    const double t278 = 3.0 * t277;
    const double t279 = t179 * pre[22];
    const double t280 = t279 - t156;
    const double t281 = pre[14] * t272;
    const double t282 = t280 + t281;
    const double t283 = t182 * pre[22];
    const double t284 = t283 - t157;
    const double t285 = pre[15] * t272;
    const double t286 = t284 + t285;
    const double t287 = t185 * pre[22];
    const double t288 = t287 - t158;
    const double t289 = pre[16] * t272;
    const double t290 = t288 + t289;
    const double t291 = t179 * pre[23];
    const double t292 = t291 - t153;
    const double t293 = pre[14] * t278;
    const double t294 = t292 + t293;
    const double t295 = t182 * pre[23];
    const double t296 = t295 - t154;
    const double t297 = pre[15] * t278;
    const double t298 = t296 + t297;
    const double t299 = t185 * pre[23];
    const double t300 = t299 - t155;
    const double t301 = pre[16] * t278;
    const double t302 = t300 + t301;
    const double t303 = t155 * t286;
    const double t304 = t154 * t290;
    const double t305 = t303 - t304;
    const double t306 = t153 * t290;
    const double t307 = t155 * t282;
    const double t308 = t306 - t307;
    const double t309 = t154 * t282;
    const double t310 = t153 * t286;
    const double t311 = t309 - t310;
    const double t312 = t158 * t298;
    const double t313 = t157 * t302;
    const double t314 = t312 - t313;
    const double t315 = t156 * t302;
    const double t316 = t158 * t294;
    const double t317 = t315 - t316;
    const double t318 = t157 * t294;
    const double t319 = t156 * t298;
    const double t320 = t318 - t319;
    const double t321 = kFA * t305;
    const double t322 = kFA * t308;
    const double t323 = kFA * t311;
    const double t324 = kFA * t314;
    const double t325 = kFA * t317;
    const double t326 = kFA * t320;
    double b244 = bout[0];
    double b249 = bout[1];
    double b254 = bout[2];
    double b324 = bout[3];
    double b325 = bout[4];
    double b326 = bout[5];
    double b321 = bout[6];
    double b322 = bout[7];
    double b323 = bout[8];
    double b320 = b326 * kFA;
    double b317 = b325 * kFA;
    double b314 = b324 * kFA;
    double b311 = b323 * kFA;
    double b308 = b322 * kFA;
    double b305 = b321 * kFA;
    double b318 = b320;
    double b319 = -b320;
    double b156 = b319 * t298;
    double b298 = b319 * t156;
    double b157 = b318 * t294;
    double b294 = b318 * t157;
    double b315 = b317;
    double b316 = -b317;
    double b158 = b316 * t294;
    b294 += b316 * t158;
    b156 += b315 * t302;
    double b302 = b315 * t156;
    double b312 = b314;
    double b313 = -b314;
    b157 += b313 * t302;
    b302 += b313 * t157;
    b158 += b312 * t298;
    b298 += b312 * t158;
    double b309 = b311;
    double b310 = -b311;
    double b153 = b310 * t286;
    double b286 = b310 * t153;
    double b154 = b309 * t282;
    double b282 = b309 * t154;
    double b306 = b308;
    double b307 = -b308;
    double b155 = b307 * t282;
    b282 += b307 * t155;
    b153 += b306 * t290;
    double b290 = b306 * t153;
    double b303 = b305;
    double b304 = -b305;
    b154 += b304 * t290;
    b290 += b304 * t154;
    b155 += b303 * t286;
    b286 += b303 * t155;
    double b300 = b302;
    double b301 = b302;
    bpre[16] += b301 * t278;
    double b278 = b301 * pre[16];
    double b299 = b300;
    b155 += -b300;
    double b185 = b299 * pre[23];
    double b296 = b298;
    double b297 = b298;
    bpre[15] += b297 * t278;
    b278 += b297 * pre[15];
    double b295 = b296;
    b154 += -b296;
    double b182 = b295 * pre[23];
    double b292 = b294;
    double b293 = b294;
    bpre[14] += b293 * t278;
    b278 += b293 * pre[14];
    double b291 = b292;
    b153 += -b292;
    double b179 = b291 * pre[23];
    double b288 = b290;
    double b289 = b290;
    bpre[16] += b289 * t272;
    double b272 = b289 * pre[16];
    double b287 = b288;
    b158 += -b288;
    b185 += b287 * pre[22];
    double b284 = b286;
    double b285 = b286;
    bpre[15] += b285 * t272;
    b272 += b285 * pre[15];
    double b283 = b284;
    b157 += -b284;
    b182 += b283 * pre[22];
    double b280 = b282;
    double b281 = b282;
    bpre[14] += b281 * t272;
    b272 += b281 * pre[14];
    double b279 = b280;
    b156 += -b280;
    b179 += b279 * pre[22];
    double b277 = b278 * 3.0;
    double b275 = b277;
    double b276 = b277;
    bpre[16] += b276 * t155;
    b155 += b276 * pre[16];
    double b273 = b275;
    double b274 = b275;
    bpre[15] += b274 * t154;
    b154 += b274 * pre[15];
    bpre[14] += b273 * t153;
    b153 += b273 * pre[14];
    double b271 = b272 * 3.0;
    double b269 = b271;
    double b270 = b271;
    bpre[16] += b270 * t158;
    b158 += b270 * pre[16];
    double b267 = b269;
    double b268 = b269;
    bpre[15] += b268 * t157;
    b157 += b268 * pre[15];
    bpre[14] += b267 * t156;
    b156 += b267 * pre[14];
    double b152 = b254;
    double b253 = b254;
    double b252 = b253 * kFA;
    double b250 = b252;
    double b251 = b252;
    double b239 = b251 * 3.0;
    double b204 = b250;
    double b230 = b250;
    double b149 = b249;
    double b248 = b249;
    double b247 = b248 * kFA;
    double b245 = b247;
    double b246 = b247;
    double b236 = b246 * 3.0;
    double b200 = b245;
    double b227 = b245;
    double b146 = b244;
    double b243 = b244;
    double b242 = b243 * kFA;
    double b240 = b242;
    double b241 = b242;
    double b233 = b241 * 3.0;
    double b196 = b240;
    double b224 = b240;
    double b237 = b239;
    double b238 = -b239;
    double b167 = b238 * t208;
    double b208 = b238 * t167;
    double b170 = b237 * t206;
    double b206 = b237 * t170;
    double b234 = b236;
    double b235 = -b236;
    double b173 = b235 * t206;
    b206 += b235 * t173;
    b167 += b234 * t210;
    double b210 = b234 * t167;
    double b231 = b233;
    double b232 = -b233;
    b170 += b232 * t210;
    b210 += b232 * t170;
    b173 += b231 * t208;
    b208 += b231 * t173;
    double b228 = b230;
    double b229 = -b230;
    double b174 = b229 * t218;
    double b218 = b229 * t174;
    double b175 = b228 * t215;
    double b215 = b228 * t175;
    double b225 = b227;
    double b226 = -b227;
    double b176 = b226 * t215;
    b215 += b226 * t176;
    b174 += b225 * t221;
    double b221 = b225 * t174;
    double b222 = b224;
    double b223 = -b224;
    b175 += b223 * t221;
    b221 += b223 * t175;
    b176 += b222 * t218;
    b218 += b222 * t176;
    double b219 = b221;
    double b220 = b221;
    bpre[16] += b220 * t211;
    double b211 = b220 * pre[16];
    b210 += b219 * 7.0;
    double b216 = b218;
    double b217 = b218;
    bpre[15] += b217 * t211;
    b211 += b217 * pre[15];
    b208 += b216 * 7.0;
    double b213 = b215;
    double b214 = b215;
    bpre[14] += b214 * t211;
    b211 += b214 * pre[14];
    b206 += b213 * 7.0;
    double b42 = b211 * 2.0;
    double b209 = b210;
    double b_hv2 = -b210;
    bpre[16] += b209 * t42;
    b42 += b209 * pre[16];
    double b207 = b208;
    double b_hv1 = -b208;
    bpre[15] += b207 * t42;
    b42 += b207 * pre[15];
    double b205 = b206;
    double b_hv0 = -b206;
    bpre[14] += b205 * t42;
    b42 += b205 * pre[14];
    bpre[21] += b204 * t203;
    double b203 = b204 * pre[21];
    b185 += b203 * t202;
    double b202 = b203 * t185;
    b173 += b202;
    double b201 = b202;
    b176 += b201 * 2.0;
    bpre[20] += b200 * t199;
    double b199 = b200 * pre[20];
    b182 += b199 * t198;
    double b198 = b199 * t182;
    b170 += b198;
    double b197 = b198;
    b175 += b197 * 2.0;
    bpre[19] += b196 * t195;
    double b195 = b196 * pre[19];
    b179 += b195 * t194;
    double b194 = b195 * t179;
    b167 += b194;
    double b193 = b194;
    b174 += b193 * 2.0;
    double b183 = b185;
    double b184 = -b185;
    bpre[1] += b184 * in_hv0;
    b_hv0 += b184 * pre[1];
    bpre[0] += b183 * in_hv1;
    b_hv1 += b183 * pre[0];
    double b180 = b182;
    double b181 = -b182;
    bpre[0] += b181 * in_hv2;
    b_hv2 += b181 * pre[0];
    bpre[2] += b180 * in_hv0;
    b_hv0 += b180 * pre[2];
    double b177 = b179;
    double b178 = -b179;
    bpre[2] += b178 * in_hv1;
    b_hv1 += b178 * pre[2];
    bpre[1] += b177 * in_hv2;
    b_hv2 += b177 * pre[1];
    b155 += b176;
    b158 += b176;
    b154 += b175;
    b157 += b175;
    b153 += b174;
    b156 += b174;
    double b171 = b173;
    double b172 = -b173;
    b155 += b172 * pre[18];
    double b_S2 = b171 * pre[17];
    double b168 = b170;
    double b169 = -b170;
    b154 += b169 * pre[18];
    double b_S1 = b168 * pre[17];
    double b165 = b167;
    double b166 = -b167;
    b153 += b166 * pre[18];
    double b_S0 = b165 * pre[17];
    b_S2 += b158 * c_moi;
    b_S1 += b157 * c_moi;
    b_S0 += b156 * c_moi;
    double b_H2 = b155 * c_hmoi;
    double b_H1 = b154 * c_hmoi;
    double b_H0 = b153 * c_hmoi;
    double b150 = b152;
    double b151 = b152;
    b_hv2 += b151 * t143;
    double b143 = b151 * in_hv2;
    bpre[16] += b150 * t138;
    double b138 = b150 * pre[16];
    double b147 = b149;
    double b148 = b149;
    b_hv1 += b148 * t143;
    b143 += b148 * in_hv1;
    bpre[15] += b147 * t138;
    b138 += b147 * pre[15];
    double b144 = b146;
    double b145 = b146;
    b_hv0 += b145 * t143;
    b143 += b145 * in_hv0;
    bpre[14] += b144 * t138;
    b138 += b144 * pre[14];
    b42 += b143 * t142;
    double b142 = b143 * t42;
    double b140 = b142;
    double b141 = b142;
    bpre[13] += b141 * t127;
    double b127 = b141 * pre[13];
    bpre[12] += b140;
    double b139 = b140;
    double b47 = b139 * pre[11];
    bpre[11] += b139 * t47;
    bpre[10] += b138 * t137;
    double b137 = b138 * pre[10];
    double b133 = b137;
    double b136 = b137;
    b127 += b136 * t135;
    double b135 = b136 * t127;
    bpre[9] += b135;
    double b134 = b135;
    b127 += b134 * pre[8];
    bpre[7] += b133;
    double b132 = b133;
    b47 += b132 * t131;
    double b131 = b132 * t47;
    double b129 = b131;
    double b130 = -b131;
    b127 += b130 * pre[6];
    bpre[5] += b129;
    double b128 = b129;
    b47 += b128 * pre[4];
    b42 += 2.0 * b127 * t42;
    double b45 = b47;
    double b46 = b47;
    b_hv2 += 2.0 * b46 * in_hv2;
    double b43 = b45;
    double b44 = b45;
    b_hv1 += 2.0 * b44 * in_hv1;
    b_hv0 += 2.0 * b43 * in_hv0;
    bpre[3] += b42 * t41;
    double b41 = b42 * pre[3];
    double b39 = b41;
    double b40 = b41;
    bpre[2] += b40 * in_hv2;
    b_hv2 += b40 * pre[2];
    double b37 = b39;
    double b38 = b39;
    bpre[1] += b38 * in_hv1;
    b_hv1 += b38 * pre[1];
    bpre[0] += b37 * in_hv0;
    b_hv0 += b37 * pre[0];
    bin[0] += b_hv0;
    bin[1] += b_hv1;
    bin[2] += b_hv2;
    bin[3] += b_S0;
    bin[4] += b_S1;
    bin[5] += b_S2;
    bin[6] += b_H0;
    bin[7] += b_H1;
    bin[8] += b_H2;
}

// adj_gr: VJP of the pre values.  bin[3] += adjoints of (x, y, z).
__host__ __device__ __forceinline__ void adj_gr_pre_vjp(double in_x, double in_y, double in_z,
        double c_hm, double c_hmg, double c_hmoi, double c_m, double c_mg, double c_moi, const double* __restrict__ bpre, double* __restrict__ bin) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t33 = 1.0 / t23;
    const double t34 = in_x * t33;
    const double t35 = in_y * t33;
    const double t36 = in_z * t33;
    const double t48 = c_mg + c_hmg;
    const double t49 = c_mg * c_hmg;
    const double t50 = t48 * t48;
    const double t51 = 1.0 / t50;
    const double t52 = t49 * t51;
    const double t53 = t23 * t23;
    const double t54 = t33 * t48;
    const double t55 = -t48;
    const double t56 = kC2 * t53;
    const double t57 = 1.0 / t56;
    const double t58 = t55 * t57;
    const double t60 = t52 * 3.0;
    const double t61 = 1.0 + t60;
    const double t63 = t52 + 2.0;
    const double t64 = 2.0 * t63;
    const double t65 = t54 * t64;
    const double t67 = t52 * 1.5;
    const double t68 = t48 * t57;
    const double t69 = 2.0 * t68;
    const double t70 = 2.0 - t52;
    const double t71 = t69 * t70;
    const double t73 = t52 * 29.0;
    const double t75 = t73 + 12.0;
    const double t77 = t75 * 0.75;
    const double t78 = 1.0 / t53;
    const double t79 = t50 * t78;
    const double t80 = t77 * t79;
    const double t82 = t52 * 4.0;
    const double t83 = 3.0 - t82;
    const double t84 = t52 * t83;
    const double t86 = t52 * 1.875;
    const double t87 = 1.0 - t60;
    const double t88 = t86 * t87;
    const double t89 = t67 * t83;
    const double t91 = t52 * 0.5;
    const double t93 = 13.0 - t82;
    const double t94 = t91 * t93;
    const double t95 = t54 * t94;
    const double t97 = t52 * 25.0;
    const double t98 = 2.0 + t97;
    const double t99 = t52 * 2.0;
    const double t100 = t52 * t99;
    const double t101 = t98 + t100;
    const double t102 = t54 * t101;
    const double t104 = t58 * -0.5;
    const double t106 = t82 + 15.0;
    const double t107 = t52 * t106;
    const double t109 = t52 * 41.0;
    const double t110 = 4.0 + t109;
    const double t112 = t52 * 8.0;
    const double t113 = t52 * t112;
    const double t114 = t110 + t113;
    const double t115 = t54 * t114;
    const double t116 = 3.0 + t99;
    const double t117 = t60 * t116;
    const double t118 = t80 - t65;
    const double t119 = t61 - t95;
    const double t120 = t67 + t102;
    const double t121 = -t120;
    const double t122 = t104 * t115;
    const double t123 = t71 - t122;
    const double t124 = t104 * t107;
    const double t125 = t104 * t117;
    const double t126 = -t125;
    const double t159 = c_hm - c_m;
    const double t160 = c_moi * t159;
    const double t161 = 1.0 / c_m;
    const double t162 = t160 * t161;
    const double t163 = 1.0 / c_hm;
    const double t164 = t159 * t163;
    const double t187 = t34 * 6.0;
    const double t188 = t33 * t187;
    const double t189 = t35 * 6.0;
    const double t190 = t33 * t189;
    const double t191 = t36 * 6.0;
    const double t192 = t33 * t191;
    const double t255 = c_m * c_hm;
    const double t256 = c_m + c_hm;
    const double t257 = 1.0 / t256;
    const double t258 = t255 * t257;
    const double t259 = c_m * 1.5;
    const double t260 = t163 * t259;
    const double t261 = 2.0 + t260;
    const double t262 = t258 * t261;
    const double t263 = c_hm * 1.5;
    const double t264 = t161 * t263;
    const double t265 = 2.0 + t264;
    const double t266 = t258 * t265;
    double b_x = bpre[0];
    double b_y = bpre[1];
    double b_z = bpre[2];
    double b33 = bpre[3];
    double b119 = bpre[5];
    double b118 = bpre[7];
    double b121 = bpre[9];
    double b58 = bpre[10];
    double b124 = bpre[11];
    double b123 = bpre[12];
    double b126 = bpre[13];
    double b34 = bpre[14];
    double b35 = bpre[15];
    double b36 = bpre[16];
    double b188 = bpre[19];
    double b190 = bpre[20];
    double b192 = bpre[21];
    b33 += b192 * t191;
    double b191 = b192 * t33;
    b36 += b191 * 6.0;
    b33 += b190 * t189;
    double b189 = b190 * t33;
    b35 += b189 * 6.0;
    b33 += b188 * t187;
    double b187 = b188 * t33;
    b34 += b187 * 6.0;
    double b125 = -b126;
    double b104 = b125 * t117;
    b104 += b124 * t107;
    double b71 = b123;
    double b122 = -b123;
    b104 += b122 * t115;
    double b115 = b122 * t104;
    double b120 = -b121;
    double b102 = b120;
    double b95 = -b119;
    double b80 = b118;
    double b65 = -b118;
    double b54 = b115 * t114;
    b58 += b104 * -0.5;
    b54 += b102 * t101;
    b54 += b95 * t94;
    double b79 = b80 * t77;
    double b78 = b79 * t50;
    double b53 = -b78 * t78 * t78;
    double b69 = b71 * t70;
    double b68 = b69 * 2.0;
    double b57 = b68 * t48;
    b54 += b65 * t64;
    b57 += b58 * t55;
    double b56 = -b57 * t57 * t57;
    b53 += b56 * kC2;
    b33 += b54 * t48;
    double b23 = 2.0 * b53 * t23;
    b_z += b36 * t33;
    b33 += b36 * in_z;
    b_y += b35 * t33;
    b33 += b35 * in_y;
    b_x += b34 * t33;
    b33 += b34 * in_x;
    b23 += -b33 * t33 * t33;
    double b22 = 0.5 * b23 / t23;
    double b20 = b22;
    double b21 = b22;
    b_z += 2.0 * b21 * in_z;
    double b18 = b20;
    double b19 = b20;
    b_y += 2.0 * b19 * in_y;
    b_x += 2.0 * b18 * in_x;
    bin[0] += b_x;
    bin[1] += b_y;
    bin[2] += b_z;
}

// adj_gr: pre values and their tangents (din[i * NT + k]: tangent k of pre input i).
template <int NT>
__host__ __device__ __forceinline__ void adj_gr_pre_jvp(double in_x, double in_y, double in_z,
        double c_hm, double c_hmg, double c_hmoi, double c_m, double c_mg, double c_moi, const double* __restrict__ din, double* __restrict__ pre,
        double* __restrict__ dpre) {
    const double t18 = in_x * in_x;
    const double t19 = in_y * in_y;
    const double t20 = t18 + t19;
    const double t21 = in_z * in_z;
    const double t22 = t20 + t21;
    const double t23 = sqrt(t22);
    const double t33 = 1.0 / t23;
    const double t34 = in_x * t33;
    const double t35 = in_y * t33;
    const double t36 = in_z * t33;
    const double t48 = c_mg + c_hmg;
    const double t49 = c_mg * c_hmg;
    const double t50 = t48 * t48;
    const double t51 = 1.0 / t50;
    const double t52 = t49 * t51;
    const double t53 = t23 * t23;
    const double t54 = t33 * t48;
    const double t55 = -t48;
    const double t56 = kC2 * t53;
    const double t57 = 1.0 / t56;
    const double t58 = t55 * t57;
    const double t60 = t52 * 3.0;
    const double t61 = 1.0 + t60;
    const double t63 = t52 + 2.0;
    const double t64 = 2.0 * t63;
    const double t65 = t54 * t64;
    const double t67 = t52 * 1.5;
    const double t68 = t48 * t57;
    const double t69 = 2.0 * t68;
    const double t70 = 2.0 - t52;
    const double t71 = t69 * t70;
    const double t73 = t52 * 29.0;
    const double t75 = t73 + 12.0;
    const double t77 = t75 * 0.75;
    const double t78 = 1.0 / t53;
    const double t79 = t50 * t78;
    const double t80 = t77 * t79;
    const double t82 = t52 * 4.0;
    const double t83 = 3.0 - t82;
    const double t84 = t52 * t83;
    const double t86 = t52 * 1.875;
    const double t87 = 1.0 - t60;
    const double t88 = t86 * t87;
    const double t89 = t67 * t83;
    const double t91 = t52 * 0.5;
    const double t93 = 13.0 - t82;
    const double t94 = t91 * t93;
    const double t95 = t54 * t94;
    const double t97 = t52 * 25.0;
    const double t98 = 2.0 + t97;
    const double t99 = t52 * 2.0;
    const double t100 = t52 * t99;
    const double t101 = t98 + t100;
    const double t102 = t54 * t101;
    const double t104 = t58 * -0.5;
    const double t106 = t82 + 15.0;
    const double t107 = t52 * t106;
    const double t109 = t52 * 41.0;
    const double t110 = 4.0 + t109;
    const double t112 = t52 * 8.0;
    const double t113 = t52 * t112;
    const double t114 = t110 + t113;
    const double t115 = t54 * t114;
    const double t116 = 3.0 + t99;
    const double t117 = t60 * t116;
    const double t118 = t80 - t65;
    const double t119 = t61 - t95;
    const double t120 = t67 + t102;
    const double t121 = -t120;
    const double t122 = t104 * t115;
    const double t123 = t71 - t122;
    const double t124 = t104 * t107;
    const double t125 = t104 * t117;
    const double t126 = -t125;
    const double t159 = c_hm - c_m;
    const double t160 = c_moi * t159;
    const double t161 = 1.0 / c_m;
    const double t162 = t160 * t161;
    const double t163 = 1.0 / c_hm;
    const double t164 = t159 * t163;
    const double t187 = t34 * 6.0;
    const double t188 = t33 * t187;
    const double t189 = t35 * 6.0;
    const double t190 = t33 * t189;
    const double t191 = t36 * 6.0;
    const double t192 = t33 * t191;
    const double t255 = c_m * c_hm;
    const double t256 = c_m + c_hm;
    const double t257 = 1.0 / t256;
    const double t258 = t255 * t257;
    const double t259 = c_m * 1.5;
    const double t260 = t163 * t259;
    const double t261 = 2.0 + t260;
    const double t262 = t258 * t261;
    const double t263 = c_hm * 1.5;
    const double t264 = t161 * t263;
    const double t265 = 2.0 + t264;
    const double t266 = t258 * t265;
    double d18[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d18[k] = 2.0 * in_x * din[0 * NT + k];
    double d19[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d19[k] = 2.0 * in_y * din[1 * NT + k];
    double d20[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d20[k] = d18[k] + d19[k];
    double d21[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d21[k] = 2.0 * in_z * din[2 * NT + k];
    double d22[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d22[k] = d20[k] + d21[k];
    double d23[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d23[k] = 0.5 * d22[k] / t23;
    double d33[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d33[k] = -t33 * t33 * d23[k];
    double d34[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d34[k] = din[0 * NT + k] * t33 + in_x * d33[k];
    double d35[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d35[k] = din[1 * NT + k] * t33 + in_y * d33[k];
    double d36[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d36[k] = din[2 * NT + k] * t33 + in_z * d33[k];
    double d53[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d53[k] = 2.0 * t23 * d23[k];
    double d54[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d54[k] = d33[k] * t48;
    double d56[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d56[k] = kC2 * d53[k];
    double d57[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d57[k] = -t57 * t57 * d56[k];
    double d58[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d58[k] = t55 * d57[k];
    double d65[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d65[k] = d54[k] * t64;
    double d68[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d68[k] = t48 * d57[k];
    double d69[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d69[k] = 2.0 * d68[k];
    double d71[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d71[k] = d69[k] * t70;
    double d78[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d78[k] = -t78 * t78 * d53[k];
    double d79[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d79[k] = t50 * d78[k];
    double d80[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d80[k] = t77 * d79[k];
    double d95[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d95[k] = d54[k] * t94;
    double d102[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d102[k] = d54[k] * t101;
    double d104[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d104[k] = d58[k] * -0.5;
    double d115[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d115[k] = d54[k] * t114;
    double d118[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d118[k] = d80[k] - d65[k];
    double d119[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d119[k] = -d95[k];
    double d120[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d120[k] = d102[k];
    double d121[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d121[k] = -d120[k];
    double d122[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d122[k] = d104[k] * t115 + t104 * d115[k];
    double d123[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d123[k] = d71[k] - d122[k];
    double d124[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d124[k] = d104[k] * t107;
    double d125[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d125[k] = d104[k] * t117;
    double d126[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d126[k] = -d125[k];
    double d187[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d187[k] = d34[k] * 6.0;
    double d188[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d188[k] = d33[k] * t187 + t33 * d187[k];
    double d189[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d189[k] = d35[k] * 6.0;
    double d190[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d190[k] = d33[k] * t189 + t33 * d189[k];
    double d191[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d191[k] = d36[k] * 6.0;
    double d192[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d192[k] = d33[k] * t191 + t33 * d191[k];
    pre[0] = in_x;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[0 * NT + k] = din[0 * NT + k];
    pre[1] = in_y;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[1 * NT + k] = din[1 * NT + k];
    pre[2] = in_z;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[2 * NT + k] = din[2 * NT + k];
    pre[3] = t33;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[3 * NT + k] = d33[k];
    pre[4] = t84;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[4 * NT + k] = 0.0;
    pre[5] = t119;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[5 * NT + k] = d119[k];
    pre[6] = t89;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[6 * NT + k] = 0.0;
    pre[7] = t118;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[7 * NT + k] = d118[k];
    pre[8] = t88;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[8 * NT + k] = 0.0;
    pre[9] = t121;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[9 * NT + k] = d121[k];
    pre[10] = t58;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[10 * NT + k] = d58[k];
    pre[11] = t124;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[11 * NT + k] = d124[k];
    pre[12] = t123;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[12 * NT + k] = d123[k];
    pre[13] = t126;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[13 * NT + k] = d126[k];
    pre[14] = t34;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[14 * NT + k] = d34[k];
    pre[15] = t35;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[15 * NT + k] = d35[k];
    pre[16] = t36;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[16 * NT + k] = d36[k];
    pre[17] = t162;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[17 * NT + k] = 0.0;
    pre[18] = t164;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[18 * NT + k] = 0.0;
    pre[19] = t188;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[19 * NT + k] = d188[k];
    pre[20] = t190;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[20 * NT + k] = d190[k];
    pre[21] = t192;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[21 * NT + k] = d192[k];
    pre[22] = t262;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[22 * NT + k] = 0.0;
    pre[23] = t266;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[23 * NT + k] = 0.0;
}

// adj_gr: one iteration, outputs and their tangents (din[i * NT + k] for the
// iteration inputs; dout[o * NT + k]).
template <int NT>
__host__ __device__ __forceinline__ void adj_gr_iter_jvp(const double* __restrict__ pre,
        const double* __restrict__ dpre, double in_hv0, double in_hv1, double in_hv2, double in_S0, double in_S1, double in_S2, double in_H0, double in_H1, double in_H2, double in_P0, double in_P1, double in_P2, double in_Q0, double in_Q1, double in_Q2,
        double c_hm, double c_hmg, double c_hmoi, double c_m, double c_mg, double c_moi, const double* __restrict__ din, double* __restrict__ out,
        double* __restrict__ dout) {
    const double t37 = pre[0] * in_hv0;
    const double t38 = pre[1] * in_hv1;
    const double t39 = t37 + t38;
    const double t40 = pre[2] * in_hv2;
    const double t41 = t39 + t40;
    const double t42 = pre[3] * t41;
    const double t43 = in_hv0 * in_hv0;
    const double t44 = in_hv1 * in_hv1;
    const double t45 = t43 + t44;
    const double t46 = in_hv2 * in_hv2;
    const double t47 = t45 + t46;
    const double t127 = t42 * t42;
    const double t128 = t47 * pre[4];
    const double t129 = pre[5] + t128;
    const double t130 = pre[6] * t127;
    const double t131 = t129 - t130;
    const double t132 = t47 * t131;
    const double t133 = pre[7] + t132;
    const double t134 = pre[8] * t127;
    const double t135 = pre[9] + t134;
    const double t136 = t127 * t135;
    const double t137 = t133 + t136;
    const double t138 = pre[10] * t137;
    const double t139 = t47 * pre[11];
    const double t140 = pre[12] + t139;
    const double t141 = pre[13] * t127;
    const double t142 = t140 + t141;
    const double t143 = t42 * t142;
    const double t144 = pre[14] * t138;
    const double t145 = in_hv0 * t143;
    const double t146 = t144 + t145;
    const double t147 = pre[15] * t138;
    const double t148 = in_hv1 * t143;
    const double t149 = t147 + t148;
    const double t150 = pre[16] * t138;
    const double t151 = in_hv2 * t143;
    const double t152 = t150 + t151;
    const double t153 = in_H0 * c_hmoi;
    const double t154 = in_H1 * c_hmoi;
    const double t155 = in_H2 * c_hmoi;
    const double t156 = in_S0 * c_moi;
    const double t157 = in_S1 * c_moi;
    const double t158 = in_S2 * c_moi;
    const double t165 = in_S0 * pre[17];
    const double t166 = t153 * pre[18];
    const double t167 = t165 - t166;
    const double t168 = in_S1 * pre[17];
    const double t169 = t154 * pre[18];
    const double t170 = t168 - t169;
    const double t171 = in_S2 * pre[17];
    const double t172 = t155 * pre[18];
    const double t173 = t171 - t172;
    const double t174 = t153 + t156;
    const double t175 = t154 + t157;
    const double t176 = t155 + t158;
    const double t177 = pre[1] * in_hv2;
    const double t178 = pre[2] * in_hv1;
    const double t179 = t177 - t178;
    const double t180 = pre[2] * in_hv0;
    const double t181 = pre[0] * in_hv2;
    const double t182 = t180 - t181;
    const double t183 = pre[0] * in_hv1;
    const double t184 = pre[1] * in_hv0;
    const double t185 = t183 - t184;
    const double t193 = 2.0 * t174;
    const double t194 = t167 + t193;
    const double t195 = t179 * t194;
    const double t196 = pre[19] * t195;
    const double t197 = 2.0 * t175;
    const double t198 = t170 + t197;
    const double t199 = t182 * t198;
    const double t200 = pre[20] * t199;
    const double t201 = 2.0 * t176;
    const double t202 = t173 + t201;
    const double t203 = t185 * t202;
    const double t204 = pre[21] * t203;
    const double t205 = pre[14] * t42;
    const double t206 = t205 - in_hv0;
    const double t207 = pre[15] * t42;
    const double t208 = t207 - in_hv1;
    const double t209 = pre[16] * t42;
    const double t210 = t209 - in_hv2;
    const double t211 = t42 * 2.0;
    const double t213 = t206 * 7.0;
    const double t214 = pre[14] * t211;
    const double t215 = t213 + t214;
    const double t216 = t208 * 7.0;
    const double t217 = pre[15] * t211;
    const double t218 = t216 + t217;
    const double t219 = t210 * 7.0;
    const double t220 = pre[16] * t211;
    const double t221 = t219 + t220;
    const double t222 = t176 * t218;
    const double t223 = t175 * t221;
    const double t224 = t222 - t223;
    const double t225 = t174 * t221;
    const double t226 = t176 * t215;
    const double t227 = t225 - t226;
    const double t228 = t175 * t215;
    const double t229 = t174 * t218;
    const double t230 = t228 - t229;
    const double t231 = t173 * t208;
    const double t232 = t170 * t210;
    const double t233 = t231 - t232;
    const double t234 = t167 * t210;
    const double t235 = t173 * t206;
    const double t236 = t234 - t235;
    const double t237 = t170 * t206;
    const double t238 = t167 * t208;
    const double t239 = t237 - t238;
    const double t240 = t196 + t224;
    const double t241 = 3.0 * t233;
    const double t242 = t240 + t241;
    const double t243 = kFA * t242;
    const double t244 = t146 + t243;
    const double t245 = t200 + t227;
    const double t246 = 3.0 * t236;
    const double t247 = t245 + t246;
    const double t248 = kFA * t247;
    const double t249 = t149 + t248;
    const double t250 = t204 + t230;
    const double t251 = 3.0 * t239;
    const double t252 = t250 + t251;
    const double t253 = kFA * t252;
    const double t254 = t152 + t253;
    const double t267 = pre[14] * t156;
    const double t268 = pre[15] * t157;
    const double t269 = t267 + t268;
    const double t270 = pre[16] * t158;
    const double t271 = t269 + t270;
    const double t272 = 3.0 * t271;
    const double t273 = pre[14] * t153;
    const double t274 = pre[15] * t154;
    const double t275 = t273 + t274;
    const double t276 = pre[16] * t155;
    const double t277 = t275 + t276;
    const double t278 = 3.0 * t277;
    const double t279 = t179 * pre[22];
    const double t280 = t279 - t156;
    const double t281 = pre[14] * t272;
    const double t282 = t280 + t281;
    const double t283 = t182 * pre[22];
    const double t284 = t283 - t157;
    const double t285 = pre[15] * t272;
    const double t286 = t284 + t285;
    const double t287 = t185 * pre[22];
    const double t288 = t287 - t158;
    const double t289 = pre[16] * t272;
    const double t290 = t288 + t289;
    const double t291 = t179 * pre[23];
    const double t292 = t291 - t153;
    const double t293 = pre[14] * t278;
    const double t294 = t292 + t293;
    const double t295 = t182 * pre[23];
    const double t296 = t295 - t154;
    const double t297 = pre[15] * t278;
    const double t298 = t296 + t297;
    const double t299 = t185 * pre[23];
    const double t300 = t299 - t155;
    const double t301 = pre[16] * t278;
    const double t302 = t300 + t301;
    const double t303 = t155 * t286;
    const double t304 = t154 * t290;
    const double t305 = t303 - t304;
    const double t306 = t153 * t290;
    const double t307 = t155 * t282;
    const double t308 = t306 - t307;
    const double t309 = t154 * t282;
    const double t310 = t153 * t286;
    const double t311 = t309 - t310;
    const double t312 = t158 * t298;
    const double t313 = t157 * t302;
    const double t314 = t312 - t313;
    const double t315 = t156 * t302;
    const double t316 = t158 * t294;
    const double t317 = t315 - t316;
    const double t318 = t157 * t294;
    const double t319 = t156 * t298;
    const double t320 = t318 - t319;
    const double t321 = kFA * t305;
    const double t322 = kFA * t308;
    const double t323 = kFA * t311;
    const double t324 = kFA * t314;
    const double t325 = kFA * t317;
    const double t326 = kFA * t320;
    double d37[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d37[k] = dpre[0 * NT + k] * in_hv0 + pre[0] * din[0 * NT + k];
    double d38[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d38[k] = dpre[1 * NT + k] * in_hv1 + pre[1] * din[1 * NT + k];
    double d39[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d39[k] = d37[k] + d38[k];
    double d40[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d40[k] = dpre[2 * NT + k] * in_hv2 + pre[2] * din[2 * NT + k];
    double d41[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d41[k] = d39[k] + d40[k];
    double d42[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d42[k] = dpre[3 * NT + k] * t41 + pre[3] * d41[k];
    double d43[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d43[k] = 2.0 * in_hv0 * din[0 * NT + k];
    double d44[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d44[k] = 2.0 * in_hv1 * din[1 * NT + k];
    double d45[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d45[k] = d43[k] + d44[k];
    double d46[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d46[k] = 2.0 * in_hv2 * din[2 * NT + k];
    double d47[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d47[k] = d45[k] + d46[k];
    double d127[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d127[k] = 2.0 * t42 * d42[k];
    double d128[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d128[k] = d47[k] * pre[4];
    double d129[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d129[k] = dpre[5 * NT + k] + d128[k];
    double d130[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d130[k] = pre[6] * d127[k];
    double d131[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d131[k] = d129[k] - d130[k];
    double d132[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d132[k] = d47[k] * t131 + t47 * d131[k];
    double d133[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d133[k] = dpre[7 * NT + k] + d132[k];
    double d134[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d134[k] = pre[8] * d127[k];
    double d135[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d135[k] = dpre[9 * NT + k] + d134[k];
    double d136[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d136[k] = d127[k] * t135 + t127 * d135[k];
    double d137[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d137[k] = d133[k] + d136[k];
    double d138[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d138[k] = dpre[10 * NT + k] * t137 + pre[10] * d137[k];
    double d139[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d139[k] = d47[k] * pre[11] + t47 * dpre[11 * NT + k];
    double d140[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d140[k] = dpre[12 * NT + k] + d139[k];
    double d141[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d141[k] = dpre[13 * NT + k] * t127 + pre[13] * d127[k];
    double d142[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d142[k] = d140[k] + d141[k];
    double d143[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d143[k] = d42[k] * t142 + t42 * d142[k];
    double d144[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d144[k] = dpre[14 * NT + k] * t138 + pre[14] * d138[k];
    double d145[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d145[k] = din[0 * NT + k] * t143 + in_hv0 * d143[k];
    double d146[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d146[k] = d144[k] + d145[k];
    double d147[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d147[k] = dpre[15 * NT + k] * t138 + pre[15] * d138[k];
    double d148[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d148[k] = din[1 * NT + k] * t143 + in_hv1 * d143[k];
    double d149[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d149[k] = d147[k] + d148[k];
    double d150[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d150[k] = dpre[16 * NT + k] * t138 + pre[16] * d138[k];
    double d151[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d151[k] = din[2 * NT + k] * t143 + in_hv2 * d143[k];
    double d152[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d152[k] = d150[k] + d151[k];
    double d153[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d153[k] = din[6 * NT + k] * c_hmoi;
    double d154[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d154[k] = din[7 * NT + k] * c_hmoi;
    double d155[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d155[k] = din[8 * NT + k] * c_hmoi;
    double d156[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d156[k] = din[3 * NT + k] * c_moi;
    double d157[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d157[k] = din[4 * NT + k] * c_moi;
    double d158[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d158[k] = din[5 * NT + k] * c_moi;
    double d165[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d165[k] = din[3 * NT + k] * pre[17];
    double d166[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d166[k] = d153[k] * pre[18];
    double d167[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d167[k] = d165[k] - d166[k];
    double d168[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d168[k] = din[4 * NT + k] * pre[17];
    double d169[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d169[k] = d154[k] * pre[18];
    double d170[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d170[k] = d168[k] - d169[k];
    double d171[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d171[k] = din[5 * NT + k] * pre[17];
    double d172[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d172[k] = d155[k] * pre[18];
    double d173[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d173[k] = d171[k] - d172[k];
    double d174[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d174[k] = d153[k] + d156[k];
    double d175[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d175[k] = d154[k] + d157[k];
    double d176[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d176[k] = d155[k] + d158[k];
    double d177[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d177[k] = dpre[1 * NT + k] * in_hv2 + pre[1] * din[2 * NT + k];
    double d178[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d178[k] = dpre[2 * NT + k] * in_hv1 + pre[2] * din[1 * NT + k];
    double d179[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d179[k] = d177[k] - d178[k];
    double d180[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d180[k] = dpre[2 * NT + k] * in_hv0 + pre[2] * din[0 * NT + k];
    double d181[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d181[k] = dpre[0 * NT + k] * in_hv2 + pre[0] * din[2 * NT + k];
    double d182[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d182[k] = d180[k] - d181[k];
    double d183[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d183[k] = dpre[0 * NT + k] * in_hv1 + pre[0] * din[1 * NT + k];
    double d184[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d184[k] = dpre[1 * NT + k] * in_hv0 + pre[1] * din[0 * NT + k];
    double d185[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d185[k] = d183[k] - d184[k];
    double d193[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d193[k] = 2.0 * d174[k];
    double d194[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d194[k] = d167[k] + d193[k];
    double d195[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d195[k] = d179[k] * t194 + t179 * d194[k];
    double d196[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d196[k] = dpre[19 * NT + k] * t195 + pre[19] * d195[k];
    double d197[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d197[k] = 2.0 * d175[k];
    double d198[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d198[k] = d170[k] + d197[k];
    double d199[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d199[k] = d182[k] * t198 + t182 * d198[k];
    double d200[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d200[k] = dpre[20 * NT + k] * t199 + pre[20] * d199[k];
    double d201[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d201[k] = 2.0 * d176[k];
    double d202[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d202[k] = d173[k] + d201[k];
    double d203[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d203[k] = d185[k] * t202 + t185 * d202[k];
    double d204[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d204[k] = dpre[21 * NT + k] * t203 + pre[21] * d203[k];
    double d205[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d205[k] = dpre[14 * NT + k] * t42 + pre[14] * d42[k];
    double d206[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d206[k] = d205[k] - din[0 * NT + k];
    double d207[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d207[k] = dpre[15 * NT + k] * t42 + pre[15] * d42[k];
    double d208[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d208[k] = d207[k] - din[1 * NT + k];
    double d209[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d209[k] = dpre[16 * NT + k] * t42 + pre[16] * d42[k];
    double d210[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d210[k] = d209[k] - din[2 * NT + k];
    double d211[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d211[k] = d42[k] * 2.0;
    double d213[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d213[k] = d206[k] * 7.0;
    double d214[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d214[k] = dpre[14 * NT + k] * t211 + pre[14] * d211[k];
    double d215[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d215[k] = d213[k] + d214[k];
    double d216[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d216[k] = d208[k] * 7.0;
    double d217[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d217[k] = dpre[15 * NT + k] * t211 + pre[15] * d211[k];
    double d218[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d218[k] = d216[k] + d217[k];
    double d219[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d219[k] = d210[k] * 7.0;
    double d220[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d220[k] = dpre[16 * NT + k] * t211 + pre[16] * d211[k];
    double d221[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d221[k] = d219[k] + d220[k];
    double d222[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d222[k] = d176[k] * t218 + t176 * d218[k];
    double d223[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d223[k] = d175[k] * t221 + t175 * d221[k];
    double d224[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d224[k] = d222[k] - d223[k];
    double d225[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d225[k] = d174[k] * t221 + t174 * d221[k];
    double d226[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d226[k] = d176[k] * t215 + t176 * d215[k];
    double d227[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d227[k] = d225[k] - d226[k];
    double d228[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d228[k] = d175[k] * t215 + t175 * d215[k];
    double d229[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d229[k] = d174[k] * t218 + t174 * d218[k];
    double d230[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d230[k] = d228[k] - d229[k];
    double d231[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d231[k] = d173[k] * t208 + t173 * d208[k];
    double d232[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d232[k] = d170[k] * t210 + t170 * d210[k];
    double d233[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d233[k] = d231[k] - d232[k];
    double d234[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d234[k] = d167[k] * t210 + t167 * d210[k];
    double d235[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d235[k] = d173[k] * t206 + t173 * d206[k];
    double d236[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d236[k] = d234[k] - d235[k];
    double d237[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d237[k] = d170[k] * t206 + t170 * d206[k];
    double d238[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d238[k] = d167[k] * t208 + t167 * d208[k];
    double d239[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d239[k] = d237[k] - d238[k];
    double d240[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d240[k] = d196[k] + d224[k];
    double d241[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d241[k] = 3.0 * d233[k];
    double d242[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d242[k] = d240[k] + d241[k];
    double d243[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d243[k] = kFA * d242[k];
    double d244[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d244[k] = d146[k] + d243[k];
    double d245[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d245[k] = d200[k] + d227[k];
    double d246[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d246[k] = 3.0 * d236[k];
    double d247[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d247[k] = d245[k] + d246[k];
    double d248[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d248[k] = kFA * d247[k];
    double d249[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d249[k] = d149[k] + d248[k];
    double d250[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d250[k] = d204[k] + d230[k];
    double d251[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d251[k] = 3.0 * d239[k];
    double d252[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d252[k] = d250[k] + d251[k];
    double d253[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d253[k] = kFA * d252[k];
    double d254[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d254[k] = d152[k] + d253[k];
    double d267[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d267[k] = dpre[14 * NT + k] * t156 + pre[14] * d156[k];
    double d268[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d268[k] = dpre[15 * NT + k] * t157 + pre[15] * d157[k];
    double d269[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d269[k] = d267[k] + d268[k];
    double d270[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d270[k] = dpre[16 * NT + k] * t158 + pre[16] * d158[k];
    double d271[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d271[k] = d269[k] + d270[k];
    double d272[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d272[k] = 3.0 * d271[k];
    double d273[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d273[k] = dpre[14 * NT + k] * t153 + pre[14] * d153[k];
    double d274[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d274[k] = dpre[15 * NT + k] * t154 + pre[15] * d154[k];
    double d275[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d275[k] = d273[k] + d274[k];
    double d276[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d276[k] = dpre[16 * NT + k] * t155 + pre[16] * d155[k];
    double d277[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d277[k] = d275[k] + d276[k];
    double d278[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d278[k] = 3.0 * d277[k];
    double d279[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d279[k] = d179[k] * pre[22];
    double d280[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d280[k] = d279[k] - d156[k];
    double d281[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d281[k] = dpre[14 * NT + k] * t272 + pre[14] * d272[k];
    double d282[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d282[k] = d280[k] + d281[k];
    double d283[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d283[k] = d182[k] * pre[22];
    double d284[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d284[k] = d283[k] - d157[k];
    double d285[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d285[k] = dpre[15 * NT + k] * t272 + pre[15] * d272[k];
    double d286[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d286[k] = d284[k] + d285[k];
    double d287[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d287[k] = d185[k] * pre[22];
    double d288[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d288[k] = d287[k] - d158[k];
    double d289[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d289[k] = dpre[16 * NT + k] * t272 + pre[16] * d272[k];
    double d290[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d290[k] = d288[k] + d289[k];
    double d291[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d291[k] = d179[k] * pre[23];
    double d292[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d292[k] = d291[k] - d153[k];
    double d293[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d293[k] = dpre[14 * NT + k] * t278 + pre[14] * d278[k];
    double d294[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d294[k] = d292[k] + d293[k];
    double d295[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d295[k] = d182[k] * pre[23];
    double d296[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d296[k] = d295[k] - d154[k];
    double d297[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d297[k] = dpre[15 * NT + k] * t278 + pre[15] * d278[k];
    double d298[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d298[k] = d296[k] + d297[k];
    double d299[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d299[k] = d185[k] * pre[23];
    double d300[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d300[k] = d299[k] - d155[k];
    double d301[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d301[k] = dpre[16 * NT + k] * t278 + pre[16] * d278[k];
    double d302[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d302[k] = d300[k] + d301[k];
    double d303[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d303[k] = d155[k] * t286 + t155 * d286[k];
    double d304[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d304[k] = d154[k] * t290 + t154 * d290[k];
    double d305[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d305[k] = d303[k] - d304[k];
    double d306[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d306[k] = d153[k] * t290 + t153 * d290[k];
    double d307[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d307[k] = d155[k] * t282 + t155 * d282[k];
    double d308[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d308[k] = d306[k] - d307[k];
    double d309[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d309[k] = d154[k] * t282 + t154 * d282[k];
    double d310[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d310[k] = d153[k] * t286 + t153 * d286[k];
    double d311[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d311[k] = d309[k] - d310[k];
    double d312[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d312[k] = d158[k] * t298 + t158 * d298[k];
    double d313[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d313[k] = d157[k] * t302 + t157 * d302[k];
    double d314[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d314[k] = d312[k] - d313[k];
    double d315[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d315[k] = d156[k] * t302 + t156 * d302[k];
    double d316[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d316[k] = d158[k] * t294 + t158 * d294[k];
    double d317[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d317[k] = d315[k] - d316[k];
    double d318[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d318[k] = d157[k] * t294 + t157 * d294[k];
    double d319[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d319[k] = d156[k] * t298 + t156 * d298[k];
    double d320[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d320[k] = d318[k] - d319[k];
    double d321[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d321[k] = kFA * d305[k];
    double d322[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d322[k] = kFA * d308[k];
    double d323[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d323[k] = kFA * d311[k];
    double d324[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d324[k] = kFA * d314[k];
    double d325[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d325[k] = kFA * d317[k];
    double d326[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d326[k] = kFA * d320[k];
    out[0] = t244;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[0 * NT + k] = d244[k];
    out[1] = t249;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[1 * NT + k] = d249[k];
    out[2] = t254;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[2 * NT + k] = d254[k];
    out[3] = t324;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[3 * NT + k] = d324[k];
    out[4] = t325;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[4 * NT + k] = d325[k];
    out[5] = t326;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[5 * NT + k] = d326[k];
    out[6] = t321;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[6 * NT + k] = d321[k];
    out[7] = t322;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[7 * NT + k] = d322[k];
    out[8] = t323;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[8 * NT + k] = d323[k];
}

}  // namespace posi_adj
