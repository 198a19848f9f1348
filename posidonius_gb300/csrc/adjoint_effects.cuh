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
    const double t83 = t82 / t65;
    const double t84 = t80 * 4.5;
    const double t85 = t84 / t65;
    const double t88 = kK2 * -3.0;
    const double t89 = t88 / t65;
    const double t90 = c_hR * t70;
    const double t91 = t67 * t90;
    const double t92 = in_k2_h * t91;
    const double t93 = c_R * t76;
    const double t94 = t68 * t93;
    const double t95 = in_k2_p * t94;
    const double t96 = t92 + t95;
    const double t97 = t89 * t96;
    const double t98 = t33 * t83;
    const double t99 = t33 * t85;
    const double t101 = -13.5 / t66;
    const double t103 = t74 + t80;
    const double t106 = t83 + t85;
    const double t107 = t33 * t106;
    const double t140 = 1.0 / c_m;
    const double t144 = t23 * t85;
    const double t145 = t23 * t83;
    pre[0] = in_x;
    pre[1] = in_y;
    pre[2] = in_z;
    pre[3] = t33;
    pre[4] = t101;
    pre[5] = t103;
    pre[6] = t97;
    pre[7] = t107;
    pre[8] = t98;
    pre[9] = t99;
    pre[10] = t34;
    pre[11] = t35;
    pre[12] = t36;
    pre[13] = t140;
    pre[14] = t85;
    pre[15] = t83;
    pre[16] = t144;
    pre[17] = t145;
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
    const double t102 = t42 * pre[4];
    const double t104 = t102 * pre[5];
    const double t105 = pre[6] + t104;
    const double t108 = t42 * pre[7];
    const double t109 = t105 + t108;
    const double t110 = in_H0 * pre[8];
    const double t111 = in_S0 * pre[9];
    const double t112 = t110 + t111;
    const double t113 = in_H1 * pre[8];
    const double t114 = in_S1 * pre[9];
    const double t115 = t113 + t114;
    const double t116 = in_H2 * pre[8];
    const double t117 = in_S2 * pre[9];
    const double t118 = t116 + t117;
    const double t119 = pre[2] * t115;
    const double t120 = pre[1] * t118;
    const double t121 = t119 - t120;
    const double t122 = pre[0] * t118;
    const double t123 = pre[2] * t112;
    const double t124 = t122 - t123;
    const double t125 = pre[1] * t112;
    const double t126 = pre[0] * t115;
    const double t127 = t125 - t126;
    const double t128 = pre[10] * t109;
    const double t129 = t121 + t128;
    const double t130 = in_hv0 * pre[7];
    const double t131 = t129 - t130;
    const double t132 = pre[11] * t109;
    const double t133 = t124 + t132;
    const double t134 = in_hv1 * pre[7];
    const double t135 = t133 - t134;
    const double t136 = pre[12] * t109;
    const double t137 = t127 + t136;
    const double t138 = in_hv2 * pre[7];
    const double t139 = t137 - t138;
    const double t141 = t131 * pre[13];
    const double t142 = t135 * pre[13];
    const double t143 = t139 * pre[13];
    const double t146 = t52 * pre[14];
    const double t147 = t47 * pre[15];
    const double t148 = in_S0 * pre[16];
    const double t149 = pre[10] * t146;
    const double t150 = t148 - t149;
    const double t151 = t55 * pre[9];
    const double t152 = t150 - t151;
    const double t153 = -t152;
    const double t154 = in_S1 * pre[16];
    const double t155 = pre[11] * t146;
    const double t156 = t154 - t155;
    const double t157 = t58 * pre[9];
    const double t158 = t156 - t157;
    const double t159 = -t158;
    const double t160 = in_S2 * pre[16];
    const double t161 = pre[12] * t146;
    const double t162 = t160 - t161;
    const double t163 = t61 * pre[9];
    const double t164 = t162 - t163;
    const double t165 = -t164;
    const double t166 = in_H0 * pre[17];
    const double t167 = pre[10] * t147;
    const double t168 = t166 - t167;
    const double t169 = t55 * pre[8];
    const double t170 = t168 - t169;
    const double t171 = -t170;
    const double t172 = in_H1 * pre[17];
    const double t173 = pre[11] * t147;
    const double t174 = t172 - t173;
    const double t175 = t58 * pre[8];
    const double t176 = t174 - t175;
    const double t177 = -t176;
    const double t178 = in_H2 * pre[17];
    const double t179 = pre[12] * t147;
    const double t180 = t178 - t179;
    const double t181 = t61 * pre[8];
    const double t182 = t180 - t181;
    const double t183 = -t182;
    out[0] = t141;
    out[1] = t142;
    out[2] = t143;
    out[3] = t153;
    out[4] = t159;
    out[5] = t165;
    out[6] = t171;
    out[7] = t177;
    out[8] = t183;
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
    const double t102 = t42 * pre[4];
    const double t104 = t102 * pre[5];
    const double t105 = pre[6] + t104;
    const double t108 = t42 * pre[7];
    const double t109 = t105 + t108;
    const double t110 = in_H0 * pre[8];
    const double t111 = in_S0 * pre[9];
    const double t112 = t110 + t111;
    const double t113 = in_H1 * pre[8];
    const double t114 = in_S1 * pre[9];
    const double t115 = t113 + t114;
    const double t116 = in_H2 * pre[8];
    const double t117 = in_S2 * pre[9];
    const double t118 = t116 + t117;
    const double t119 = pre[2] * t115;
    const double t120 = pre[1] * t118;
    const double t121 = t119 - t120;
    const double t122 = pre[0] * t118;
    const double t123 = pre[2] * t112;
    const double t124 = t122 - t123;
    const double t125 = pre[1] * t112;
    const double t126 = pre[0] * t115;
    const double t127 = t125 - t126;
    const double t128 = pre[10] * t109;
    const double t129 = t121 + t128;
    const double t130 = in_hv0 * pre[7];
    const double t131 = t129 - t130;
    const double t132 = pre[11] * t109;
    const double t133 = t124 + t132;
    const double t134 = in_hv1 * pre[7];
    const double t135 = t133 - t134;
    const double t136 = pre[12] * t109;
    const double t137 = t127 + t136;
    const double t138 = in_hv2 * pre[7];
    const double t139 = t137 - t138;
    const double t141 = t131 * pre[13];
    const double t142 = t135 * pre[13];
    const double t143 = t139 * pre[13];
    const double t146 = t52 * pre[14];
    const double t147 = t47 * pre[15];
    const double t148 = in_S0 * pre[16];
    const double t149 = pre[10] * t146;
    const double t150 = t148 - t149;
    const double t151 = t55 * pre[9];
    const double t152 = t150 - t151;
    const double t153 = -t152;
    const double t154 = in_S1 * pre[16];
    const double t155 = pre[11] * t146;
    const double t156 = t154 - t155;
    const double t157 = t58 * pre[9];
    const double t158 = t156 - t157;
    const double t159 = -t158;
    const double t160 = in_S2 * pre[16];
    const double t161 = pre[12] * t146;
    const double t162 = t160 - t161;
    const double t163 = t61 * pre[9];
    const double t164 = t162 - t163;
    const double t165 = -t164;
    const double t166 = in_H0 * pre[17];
    const double t167 = pre[10] * t147;
    const double t168 = t166 - t167;
    const double t169 = t55 * pre[8];
    const double t170 = t168 - t169;
    const double t171 = -t170;
    const double t172 = in_H1 * pre[17];
    const double t173 = pre[11] * t147;
    const double t174 = t172 - t173;
    const double t175 = t58 * pre[8];
    const double t176 = t174 - t175;
    const double t177 = -t176;
    const double t178 = in_H2 * pre[17];
    const double t179 = pre[12] * t147;
    const double t180 = t178 - t179;
    const double t181 = t61 * pre[8];
    const double t182 = t180 - t181;
    const double t183 = -t182;
    double b141 = bout[0];
    double b142 = bout[1];
    double b143 = bout[2];
    double b153 = bout[3];
    double b159 = bout[4];
    double b165 = bout[5];
    double b171 = bout[6];
    double b177 = bout[7];
    double b183 = bout[8];
    double b182 = -b183;
    double b180 = b182;
    double b181 = -b182;
    double b61 = b181 * pre[8];
    bpre[8] += b181 * t61;
    double b178 = b180;
    double b179 = -b180;
    bpre[12] += b179 * t147;
    double b147 = b179 * pre[12];
    double b_H2 = b178 * pre[17];
    bpre[17] += b178 * in_H2;
    double b176 = -b177;
    double b174 = b176;
    double b175 = -b176;
    double b58 = b175 * pre[8];
    bpre[8] += b175 * t58;
    double b172 = b174;
    double b173 = -b174;
    bpre[11] += b173 * t147;
    b147 += b173 * pre[11];
    double b_H1 = b172 * pre[17];
    bpre[17] += b172 * in_H1;
    double b170 = -b171;
    double b168 = b170;
    double b169 = -b170;
    double b55 = b169 * pre[8];
    bpre[8] += b169 * t55;
    double b166 = b168;
    double b167 = -b168;
    bpre[10] += b167 * t147;
    b147 += b167 * pre[10];
    double b_H0 = b166 * pre[17];
    bpre[17] += b166 * in_H0;
    double b164 = -b165;
    double b162 = b164;
    double b163 = -b164;
    b61 += b163 * pre[9];
    bpre[9] += b163 * t61;
    double b160 = b162;
    double b161 = -b162;
    bpre[12] += b161 * t146;
    double b146 = b161 * pre[12];
    double b_S2 = b160 * pre[16];
    bpre[16] += b160 * in_S2;
    double b158 = -b159;
    double b156 = b158;
    double b157 = -b158;
    b58 += b157 * pre[9];
    bpre[9] += b157 * t58;
    double b154 = b156;
    double b155 = -b156;
    bpre[11] += b155 * t146;
    b146 += b155 * pre[11];
    double b_S1 = b154 * pre[16];
    bpre[16] += b154 * in_S1;
    double b152 = -b153;
    double b150 = b152;
    double b151 = -b152;
    b55 += b151 * pre[9];
    bpre[9] += b151 * t55;
    double b148 = b150;
    double b149 = -b150;
    bpre[10] += b149 * t146;
    b146 += b149 * pre[10];
    double b_S0 = b148 * pre[16];
    bpre[16] += b148 * in_S0;
    double b47 = b147 * pre[15];
    bpre[15] += b147 * t47;
    double b52 = b146 * pre[14];
    bpre[14] += b146 * t52;
    double b139 = b143 * pre[13];
    double b135 = b142 * pre[13];
    double b131 = b141 * pre[13];
    double b137 = b139;
    double b138 = -b139;
    double b_hv2 = b138 * pre[7];
    bpre[7] += b138 * in_hv2;
    double b127 = b137;
    double b136 = b137;
    bpre[12] += b136 * t109;
    double b109 = b136 * pre[12];
    double b133 = b135;
    double b134 = -b135;
    double b_hv1 = b134 * pre[7];
    bpre[7] += b134 * in_hv1;
    double b124 = b133;
    double b132 = b133;
    bpre[11] += b132 * t109;
    b109 += b132 * pre[11];
    double b129 = b131;
    double b130 = -b131;
    double b_hv0 = b130 * pre[7];
    bpre[7] += b130 * in_hv0;
    double b121 = b129;
    double b128 = b129;
    bpre[10] += b128 * t109;
    b109 += b128 * pre[10];
    double b125 = b127;
    double b126 = -b127;
    bpre[0] += b126 * t115;
    double b115 = b126 * pre[0];
    bpre[1] += b125 * t112;
    double b112 = b125 * pre[1];
    double b122 = b124;
    double b123 = -b124;
    bpre[2] += b123 * t112;
    b112 += b123 * pre[2];
    bpre[0] += b122 * t118;
    double b118 = b122 * pre[0];
    double b119 = b121;
    double b120 = -b121;
    bpre[1] += b120 * t118;
    b118 += b120 * pre[1];
    bpre[2] += b119 * t115;
    b115 += b119 * pre[2];
    double b116 = b118;
    double b117 = b118;
    b_S2 += b117 * pre[9];
    bpre[9] += b117 * in_S2;
    b_H2 += b116 * pre[8];
    bpre[8] += b116 * in_H2;
    double b113 = b115;
    double b114 = b115;
    b_S1 += b114 * pre[9];
    bpre[9] += b114 * in_S1;
    b_H1 += b113 * pre[8];
    bpre[8] += b113 * in_H1;
    double b110 = b112;
    double b111 = b112;
    b_S0 += b111 * pre[9];
    bpre[9] += b111 * in_S0;
    b_H0 += b110 * pre[8];
    bpre[8] += b110 * in_H0;
    double b105 = b109;
    double b108 = b109;
    double b42 = b108 * pre[7];
    bpre[7] += b108 * t42;
    bpre[6] += b105;
    double b104 = b105;
    double b102 = b104 * pre[5];
    bpre[5] += b104 * t102;
    b42 += b102 * pre[4];
    bpre[4] += b102 * t42;
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
    const double t83 = t82 / t65;
    const double t84 = t80 * 4.5;
    const double t85 = t84 / t65;
    const double t88 = kK2 * -3.0;
    const double t89 = t88 / t65;
    const double t90 = c_hR * t70;
    const double t91 = t67 * t90;
    const double t92 = in_k2_h * t91;
    const double t93 = c_R * t76;
    const double t94 = t68 * t93;
    const double t95 = in_k2_p * t94;
    const double t96 = t92 + t95;
    const double t97 = t89 * t96;
    const double t98 = t33 * t83;
    const double t99 = t33 * t85;
    const double t101 = -13.5 / t66;
    const double t103 = t74 + t80;
    const double t106 = t83 + t85;
    const double t107 = t33 * t106;
    const double t140 = 1.0 / c_m;
    const double t144 = t23 * t85;
    const double t145 = t23 * t83;
    double b_x = bpre[0];
    double b_y = bpre[1];
    double b_z = bpre[2];
    double b33 = bpre[3];
    double b101 = bpre[4];
    double b103 = bpre[5];
    double b97 = bpre[6];
    double b107 = bpre[7];
    double b98 = bpre[8];
    double b99 = bpre[9];
    double b34 = bpre[10];
    double b35 = bpre[11];
    double b36 = bpre[12];
    double b85 = bpre[14];
    double b83 = bpre[15];
    double b144 = bpre[16];
    double b145 = bpre[17];
    double b23 = b145 * t83;
    b83 += b145 * t23;
    b23 += b144 * t85;
    b85 += b144 * t23;
    b33 += b107 * t106;
    double b106 = b107 * t33;
    b83 += b106;
    b85 += b106;
    double b74 = b103;
    double b80 = b103;
    double b66 = -b101 * t101 / t66;
    b33 += b99 * t85;
    b85 += b99 * t33;
    b33 += b98 * t83;
    b83 += b98 * t33;
    double b89 = b97 * t96;
    double b96 = b97 * t89;
    double b92 = b96;
    double b95 = b96;
    double b_k2_p = b95 * t94;
    double b_k2_h = b92 * t91;
    double b65 = -b89 * t89 / t65;
    double b84 = b85 / t65;
    b65 += -b85 * t85 / t65;
    b80 += b84 * 4.5;
    double b82 = b83 / t65;
    b65 += -b83 * t83 / t65;
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
    b23 += -b33 * t33 / t23;
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
    const double t83 = t82 / t65;
    const double t84 = t80 * 4.5;
    const double t85 = t84 / t65;
    const double t88 = kK2 * -3.0;
    const double t89 = t88 / t65;
    const double t90 = c_hR * t70;
    const double t91 = t67 * t90;
    const double t92 = in_k2_h * t91;
    const double t93 = c_R * t76;
    const double t94 = t68 * t93;
    const double t95 = in_k2_p * t94;
    const double t96 = t92 + t95;
    const double t97 = t89 * t96;
    const double t98 = t33 * t83;
    const double t99 = t33 * t85;
    const double t101 = -13.5 / t66;
    const double t103 = t74 + t80;
    const double t106 = t83 + t85;
    const double t107 = t33 * t106;
    const double t140 = 1.0 / c_m;
    const double t144 = t23 * t85;
    const double t145 = t23 * t83;
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
    for (int k = 0; k < NT; ++k) d33[k] = -t33 * d23[k] / t23;
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
    for (int k = 0; k < NT; ++k) d83[k] = (d82[k] - t83 * d65[k]) / t65;
    double d84[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d84[k] = d80[k] * 4.5;
    double d85[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d85[k] = (d84[k] - t85 * d65[k]) / t65;
    double d89[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d89[k] = -t89 * d65[k] / t65;
    double d92[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d92[k] = din[6 * NT + k] * t91;
    double d95[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d95[k] = din[5 * NT + k] * t94;
    double d96[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d96[k] = d92[k] + d95[k];
    double d97[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d97[k] = d89[k] * t96 + t89 * d96[k];
    double d98[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d98[k] = d33[k] * t83 + t33 * d83[k];
    double d99[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d99[k] = d33[k] * t85 + t33 * d85[k];
    double d101[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d101[k] = -t101 * d66[k] / t66;
    double d103[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d103[k] = d74[k] + d80[k];
    double d106[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d106[k] = d83[k] + d85[k];
    double d107[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d107[k] = d33[k] * t106 + t33 * d106[k];
    double d144[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d144[k] = d23[k] * t85 + t23 * d85[k];
    double d145[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d145[k] = d23[k] * t83 + t23 * d83[k];
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
    pre[4] = t101;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[4 * NT + k] = d101[k];
    pre[5] = t103;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[5 * NT + k] = d103[k];
    pre[6] = t97;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[6 * NT + k] = d97[k];
    pre[7] = t107;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[7 * NT + k] = d107[k];
    pre[8] = t98;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[8 * NT + k] = d98[k];
    pre[9] = t99;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[9 * NT + k] = d99[k];
    pre[10] = t34;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[10 * NT + k] = d34[k];
    pre[11] = t35;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[11 * NT + k] = d35[k];
    pre[12] = t36;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[12 * NT + k] = d36[k];
    pre[13] = t140;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[13 * NT + k] = 0.0;
    pre[14] = t85;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[14 * NT + k] = d85[k];
    pre[15] = t83;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[15 * NT + k] = d83[k];
    pre[16] = t144;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[16 * NT + k] = d144[k];
    pre[17] = t145;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[17 * NT + k] = d145[k];
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
    const double t102 = t42 * pre[4];
    const double t104 = t102 * pre[5];
    const double t105 = pre[6] + t104;
    const double t108 = t42 * pre[7];
    const double t109 = t105 + t108;
    const double t110 = in_H0 * pre[8];
    const double t111 = in_S0 * pre[9];
    const double t112 = t110 + t111;
    const double t113 = in_H1 * pre[8];
    const double t114 = in_S1 * pre[9];
    const double t115 = t113 + t114;
    const double t116 = in_H2 * pre[8];
    const double t117 = in_S2 * pre[9];
    const double t118 = t116 + t117;
    const double t119 = pre[2] * t115;
    const double t120 = pre[1] * t118;
    const double t121 = t119 - t120;
    const double t122 = pre[0] * t118;
    const double t123 = pre[2] * t112;
    const double t124 = t122 - t123;
    const double t125 = pre[1] * t112;
    const double t126 = pre[0] * t115;
    const double t127 = t125 - t126;
    const double t128 = pre[10] * t109;
    const double t129 = t121 + t128;
    const double t130 = in_hv0 * pre[7];
    const double t131 = t129 - t130;
    const double t132 = pre[11] * t109;
    const double t133 = t124 + t132;
    const double t134 = in_hv1 * pre[7];
    const double t135 = t133 - t134;
    const double t136 = pre[12] * t109;
    const double t137 = t127 + t136;
    const double t138 = in_hv2 * pre[7];
    const double t139 = t137 - t138;
    const double t141 = t131 * pre[13];
    const double t142 = t135 * pre[13];
    const double t143 = t139 * pre[13];
    const double t146 = t52 * pre[14];
    const double t147 = t47 * pre[15];
    const double t148 = in_S0 * pre[16];
    const double t149 = pre[10] * t146;
    const double t150 = t148 - t149;
    const double t151 = t55 * pre[9];
    const double t152 = t150 - t151;
    const double t153 = -t152;
    const double t154 = in_S1 * pre[16];
    const double t155 = pre[11] * t146;
    const double t156 = t154 - t155;
    const double t157 = t58 * pre[9];
    const double t158 = t156 - t157;
    const double t159 = -t158;
    const double t160 = in_S2 * pre[16];
    const double t161 = pre[12] * t146;
    const double t162 = t160 - t161;
    const double t163 = t61 * pre[9];
    const double t164 = t162 - t163;
    const double t165 = -t164;
    const double t166 = in_H0 * pre[17];
    const double t167 = pre[10] * t147;
    const double t168 = t166 - t167;
    const double t169 = t55 * pre[8];
    const double t170 = t168 - t169;
    const double t171 = -t170;
    const double t172 = in_H1 * pre[17];
    const double t173 = pre[11] * t147;
    const double t174 = t172 - t173;
    const double t175 = t58 * pre[8];
    const double t176 = t174 - t175;
    const double t177 = -t176;
    const double t178 = in_H2 * pre[17];
    const double t179 = pre[12] * t147;
    const double t180 = t178 - t179;
    const double t181 = t61 * pre[8];
    const double t182 = t180 - t181;
    const double t183 = -t182;
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
    double d102[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d102[k] = d42[k] * pre[4] + t42 * dpre[4 * NT + k];
    double d104[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d104[k] = d102[k] * pre[5] + t102 * dpre[5 * NT + k];
    double d105[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d105[k] = dpre[6 * NT + k] + d104[k];
    double d108[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d108[k] = d42[k] * pre[7] + t42 * dpre[7 * NT + k];
    double d109[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d109[k] = d105[k] + d108[k];
    double d110[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d110[k] = din[6 * NT + k] * pre[8] + in_H0 * dpre[8 * NT + k];
    double d111[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d111[k] = din[3 * NT + k] * pre[9] + in_S0 * dpre[9 * NT + k];
    double d112[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d112[k] = d110[k] + d111[k];
    double d113[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d113[k] = din[7 * NT + k] * pre[8] + in_H1 * dpre[8 * NT + k];
    double d114[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d114[k] = din[4 * NT + k] * pre[9] + in_S1 * dpre[9 * NT + k];
    double d115[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d115[k] = d113[k] + d114[k];
    double d116[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d116[k] = din[8 * NT + k] * pre[8] + in_H2 * dpre[8 * NT + k];
    double d117[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d117[k] = din[5 * NT + k] * pre[9] + in_S2 * dpre[9 * NT + k];
    double d118[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d118[k] = d116[k] + d117[k];
    double d119[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d119[k] = dpre[2 * NT + k] * t115 + pre[2] * d115[k];
    double d120[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d120[k] = dpre[1 * NT + k] * t118 + pre[1] * d118[k];
    double d121[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d121[k] = d119[k] - d120[k];
    double d122[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d122[k] = dpre[0 * NT + k] * t118 + pre[0] * d118[k];
    double d123[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d123[k] = dpre[2 * NT + k] * t112 + pre[2] * d112[k];
    double d124[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d124[k] = d122[k] - d123[k];
    double d125[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d125[k] = dpre[1 * NT + k] * t112 + pre[1] * d112[k];
    double d126[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d126[k] = dpre[0 * NT + k] * t115 + pre[0] * d115[k];
    double d127[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d127[k] = d125[k] - d126[k];
    double d128[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d128[k] = dpre[10 * NT + k] * t109 + pre[10] * d109[k];
    double d129[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d129[k] = d121[k] + d128[k];
    double d130[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d130[k] = din[0 * NT + k] * pre[7] + in_hv0 * dpre[7 * NT + k];
    double d131[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d131[k] = d129[k] - d130[k];
    double d132[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d132[k] = dpre[11 * NT + k] * t109 + pre[11] * d109[k];
    double d133[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d133[k] = d124[k] + d132[k];
    double d134[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d134[k] = din[1 * NT + k] * pre[7] + in_hv1 * dpre[7 * NT + k];
    double d135[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d135[k] = d133[k] - d134[k];
    double d136[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d136[k] = dpre[12 * NT + k] * t109 + pre[12] * d109[k];
    double d137[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d137[k] = d127[k] + d136[k];
    double d138[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d138[k] = din[2 * NT + k] * pre[7] + in_hv2 * dpre[7 * NT + k];
    double d139[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d139[k] = d137[k] - d138[k];
    double d141[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d141[k] = d131[k] * pre[13];
    double d142[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d142[k] = d135[k] * pre[13];
    double d143[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d143[k] = d139[k] * pre[13];
    double d146[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d146[k] = d52[k] * pre[14] + t52 * dpre[14 * NT + k];
    double d147[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d147[k] = d47[k] * pre[15] + t47 * dpre[15 * NT + k];
    double d148[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d148[k] = din[3 * NT + k] * pre[16] + in_S0 * dpre[16 * NT + k];
    double d149[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d149[k] = dpre[10 * NT + k] * t146 + pre[10] * d146[k];
    double d150[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d150[k] = d148[k] - d149[k];
    double d151[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d151[k] = d55[k] * pre[9] + t55 * dpre[9 * NT + k];
    double d152[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d152[k] = d150[k] - d151[k];
    double d153[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d153[k] = -d152[k];
    double d154[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d154[k] = din[4 * NT + k] * pre[16] + in_S1 * dpre[16 * NT + k];
    double d155[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d155[k] = dpre[11 * NT + k] * t146 + pre[11] * d146[k];
    double d156[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d156[k] = d154[k] - d155[k];
    double d157[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d157[k] = d58[k] * pre[9] + t58 * dpre[9 * NT + k];
    double d158[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d158[k] = d156[k] - d157[k];
    double d159[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d159[k] = -d158[k];
    double d160[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d160[k] = din[5 * NT + k] * pre[16] + in_S2 * dpre[16 * NT + k];
    double d161[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d161[k] = dpre[12 * NT + k] * t146 + pre[12] * d146[k];
    double d162[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d162[k] = d160[k] - d161[k];
    double d163[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d163[k] = d61[k] * pre[9] + t61 * dpre[9 * NT + k];
    double d164[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d164[k] = d162[k] - d163[k];
    double d165[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d165[k] = -d164[k];
    double d166[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d166[k] = din[6 * NT + k] * pre[17] + in_H0 * dpre[17 * NT + k];
    double d167[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d167[k] = dpre[10 * NT + k] * t147 + pre[10] * d147[k];
    double d168[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d168[k] = d166[k] - d167[k];
    double d169[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d169[k] = d55[k] * pre[8] + t55 * dpre[8 * NT + k];
    double d170[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d170[k] = d168[k] - d169[k];
    double d171[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d171[k] = -d170[k];
    double d172[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d172[k] = din[7 * NT + k] * pre[17] + in_H1 * dpre[17 * NT + k];
    double d173[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d173[k] = dpre[11 * NT + k] * t147 + pre[11] * d147[k];
    double d174[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d174[k] = d172[k] - d173[k];
    double d175[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d175[k] = d58[k] * pre[8] + t58 * dpre[8 * NT + k];
    double d176[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d176[k] = d174[k] - d175[k];
    double d177[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d177[k] = -d176[k];
    double d178[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d178[k] = din[8 * NT + k] * pre[17] + in_H2 * dpre[17 * NT + k];
    double d179[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d179[k] = dpre[12 * NT + k] * t147 + pre[12] * d147[k];
    double d180[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d180[k] = d178[k] - d179[k];
    double d181[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d181[k] = d61[k] * pre[8] + t61 * dpre[8 * NT + k];
    double d182[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d182[k] = d180[k] - d181[k];
    double d183[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d183[k] = -d182[k];
    out[0] = t141;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[0 * NT + k] = d141[k];
    out[1] = t142;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[1 * NT + k] = d142[k];
    out[2] = t143;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[2 * NT + k] = d143[k];
    out[3] = t153;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[3 * NT + k] = d153[k];
    out[4] = t159;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[4 * NT + k] = d159[k];
    out[5] = t165;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[5 * NT + k] = d165[k];
    out[6] = t171;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[6 * NT + k] = d171[k];
    out[7] = t177;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[7 * NT + k] = d177[k];
    out[8] = t183;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[8 * NT + k] = d183[k];
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
    const double t78 = -3.0 / t55;
    const double t84 = 15.0 / t57;
    const double t107 = 1.0 / c_m;
    pre[0] = in_x;
    pre[1] = in_y;
    pre[2] = in_z;
    pre[3] = t62;
    pre[4] = t65;
    pre[5] = t52;
    pre[6] = t46;
    pre[7] = t78;
    pre[8] = t84;
    pre[9] = t107;
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
    const double t85 = t34 * pre[6];
    const double t86 = t34 * t85;
    const double t87 = t39 * pre[5];
    const double t88 = t39 * t87;
    const double t89 = t86 + t88;
    const double t90 = pre[8] * t89;
    const double t91 = t82 + t90;
    const double t92 = pre[0] * t91;
    const double t93 = in_S0 * t66;
    const double t94 = t92 + t93;
    const double t95 = in_H0 * t63;
    const double t96 = t94 + t95;
    const double t97 = pre[1] * t91;
    const double t98 = in_S1 * t66;
    const double t99 = t97 + t98;
    const double t100 = in_H1 * t63;
    const double t101 = t99 + t100;
    const double t102 = pre[2] * t91;
    const double t103 = in_S2 * t66;
    const double t104 = t102 + t103;
    const double t105 = in_H2 * t63;
    const double t106 = t104 + t105;
    const double t108 = t96 * pre[9];
    const double t109 = t101 * pre[9];
    const double t110 = t106 * pre[9];
    const double t111 = pre[1] * in_S2;
    const double t112 = pre[2] * in_S1;
    const double t113 = t111 - t112;
    const double t114 = pre[2] * in_S0;
    const double t115 = pre[0] * in_S2;
    const double t116 = t114 - t115;
    const double t117 = pre[0] * in_S1;
    const double t118 = pre[1] * in_S0;
    const double t119 = t117 - t118;
    const double t120 = pre[1] * in_H2;
    const double t121 = pre[2] * in_H1;
    const double t122 = t120 - t121;
    const double t123 = pre[2] * in_H0;
    const double t124 = pre[0] * in_H2;
    const double t125 = t123 - t124;
    const double t126 = pre[0] * in_H1;
    const double t127 = pre[1] * in_H0;
    const double t128 = t126 - t127;
    const double t129 = t66 * t113;
    const double t130 = -t129;
    const double t131 = t66 * t116;
    const double t132 = -t131;
    const double t133 = t66 * t119;
    const double t134 = -t133;
    const double t135 = t63 * t122;
    const double t136 = -t135;
    const double t137 = t63 * t125;
    const double t138 = -t137;
    const double t139 = t63 * t128;
    const double t140 = -t139;
    out[0] = t108;
    out[1] = t109;
    out[2] = t110;
    out[3] = t130;
    out[4] = t132;
    out[5] = t134;
    out[6] = t136;
    out[7] = t138;
    out[8] = t140;
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
    const double t85 = t34 * pre[6];
    const double t86 = t34 * t85;
    const double t87 = t39 * pre[5];
    const double t88 = t39 * t87;
    const double t89 = t86 + t88;
    const double t90 = pre[8] * t89;
    const double t91 = t82 + t90;
    const double t92 = pre[0] * t91;
    const double t93 = in_S0 * t66;
    const double t94 = t92 + t93;
    const double t95 = in_H0 * t63;
    const double t96 = t94 + t95;
    const double t97 = pre[1] * t91;
    const double t98 = in_S1 * t66;
    const double t99 = t97 + t98;
    const double t100 = in_H1 * t63;
    const double t101 = t99 + t100;
    const double t102 = pre[2] * t91;
    const double t103 = in_S2 * t66;
    const double t104 = t102 + t103;
    const double t105 = in_H2 * t63;
    const double t106 = t104 + t105;
    const double t108 = t96 * pre[9];
    const double t109 = t101 * pre[9];
    const double t110 = t106 * pre[9];
    const double t111 = pre[1] * in_S2;
    const double t112 = pre[2] * in_S1;
    const double t113 = t111 - t112;
    const double t114 = pre[2] * in_S0;
    const double t115 = pre[0] * in_S2;
    const double t116 = t114 - t115;
    const double t117 = pre[0] * in_S1;
    const double t118 = pre[1] * in_S0;
    const double t119 = t117 - t118;
    const double t120 = pre[1] * in_H2;
    const double t121 = pre[2] * in_H1;
    const double t122 = t120 - t121;
    const double t123 = pre[2] * in_H0;
    const double t124 = pre[0] * in_H2;
    const double t125 = t123 - t124;
    const double t126 = pre[0] * in_H1;
    const double t127 = pre[1] * in_H0;
    const double t128 = t126 - t127;
    const double t129 = t66 * t113;
    const double t130 = -t129;
    const double t131 = t66 * t116;
    const double t132 = -t131;
    const double t133 = t66 * t119;
    const double t134 = -t133;
    const double t135 = t63 * t122;
    const double t136 = -t135;
    const double t137 = t63 * t125;
    const double t138 = -t137;
    const double t139 = t63 * t128;
    const double t140 = -t139;
    double b108 = bout[0];
    double b109 = bout[1];
    double b110 = bout[2];
    double b130 = bout[3];
    double b132 = bout[4];
    double b134 = bout[5];
    double b136 = bout[6];
    double b138 = bout[7];
    double b140 = bout[8];
    double b139 = -b140;
    double b63 = b139 * t128;
    double b128 = b139 * t63;
    double b137 = -b138;
    b63 += b137 * t125;
    double b125 = b137 * t63;
    double b135 = -b136;
    b63 += b135 * t122;
    double b122 = b135 * t63;
    double b133 = -b134;
    double b66 = b133 * t119;
    double b119 = b133 * t66;
    double b131 = -b132;
    b66 += b131 * t116;
    double b116 = b131 * t66;
    double b129 = -b130;
    b66 += b129 * t113;
    double b113 = b129 * t66;
    double b126 = b128;
    double b127 = -b128;
    bpre[1] += b127 * in_H0;
    double b_H0 = b127 * pre[1];
    bpre[0] += b126 * in_H1;
    double b_H1 = b126 * pre[0];
    double b123 = b125;
    double b124 = -b125;
    bpre[0] += b124 * in_H2;
    double b_H2 = b124 * pre[0];
    bpre[2] += b123 * in_H0;
    b_H0 += b123 * pre[2];
    double b120 = b122;
    double b121 = -b122;
    bpre[2] += b121 * in_H1;
    b_H1 += b121 * pre[2];
    bpre[1] += b120 * in_H2;
    b_H2 += b120 * pre[1];
    double b117 = b119;
    double b118 = -b119;
    bpre[1] += b118 * in_S0;
    double b_S0 = b118 * pre[1];
    bpre[0] += b117 * in_S1;
    double b_S1 = b117 * pre[0];
    double b114 = b116;
    double b115 = -b116;
    bpre[0] += b115 * in_S2;
    double b_S2 = b115 * pre[0];
    bpre[2] += b114 * in_S0;
    b_S0 += b114 * pre[2];
    double b111 = b113;
    double b112 = -b113;
    bpre[2] += b112 * in_S1;
    b_S1 += b112 * pre[2];
    bpre[1] += b111 * in_S2;
    b_S2 += b111 * pre[1];
    double b106 = b110 * pre[9];
    double b101 = b109 * pre[9];
    double b96 = b108 * pre[9];
    double b104 = b106;
    double b105 = b106;
    b_H2 += b105 * t63;
    b63 += b105 * in_H2;
    double b102 = b104;
    double b103 = b104;
    b_S2 += b103 * t66;
    b66 += b103 * in_S2;
    bpre[2] += b102 * t91;
    double b91 = b102 * pre[2];
    double b99 = b101;
    double b100 = b101;
    b_H1 += b100 * t63;
    b63 += b100 * in_H1;
    double b97 = b99;
    double b98 = b99;
    b_S1 += b98 * t66;
    b66 += b98 * in_S1;
    bpre[1] += b97 * t91;
    b91 += b97 * pre[1];
    double b94 = b96;
    double b95 = b96;
    b_H0 += b95 * t63;
    b63 += b95 * in_H0;
    double b92 = b94;
    double b93 = b94;
    b_S0 += b93 * t66;
    b66 += b93 * in_S0;
    bpre[0] += b92 * t91;
    b91 += b92 * pre[0];
    double b82 = b91;
    double b90 = b91;
    bpre[8] += b90 * t89;
    double b89 = b90 * pre[8];
    double b86 = b89;
    double b88 = b89;
    double b39 = b88 * t87;
    double b87 = b88 * t39;
    b39 += b87 * pre[5];
    double b34 = b86 * t85;
    double b85 = b86 * t34;
    b34 += b85 * pre[6];
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
    const double t78 = -3.0 / t55;
    const double t84 = 15.0 / t57;
    const double t107 = 1.0 / c_m;
    double b_x = bpre[0];
    double b_y = bpre[1];
    double b_z = bpre[2];
    double b62 = bpre[3];
    double b65 = bpre[4];
    double b78 = bpre[7];
    double b84 = bpre[8];
    double b57 = -b84 * t84 / t57;
    double b55 = -b78 * t78 / t55;
    double b59 = b65 * t64;
    b59 += b62 * t61;
    b55 += -b59 * t59 / t55;
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
    const double t78 = -3.0 / t55;
    const double t84 = 15.0 / t57;
    const double t107 = 1.0 / c_m;
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
    for (int k = 0; k < NT; ++k) d59[k] = -t59 * d55[k] / t55;
    double d62[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d62[k] = d59[k] * t61;
    double d65[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d65[k] = d59[k] * t64;
    double d78[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d78[k] = -t78 * d55[k] / t55;
    double d84[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d84[k] = -t84 * d57[k] / t57;
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
    pre[8] = t84;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[8 * NT + k] = d84[k];
    pre[9] = t107;
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
    const double t85 = t34 * pre[6];
    const double t86 = t34 * t85;
    const double t87 = t39 * pre[5];
    const double t88 = t39 * t87;
    const double t89 = t86 + t88;
    const double t90 = pre[8] * t89;
    const double t91 = t82 + t90;
    const double t92 = pre[0] * t91;
    const double t93 = in_S0 * t66;
    const double t94 = t92 + t93;
    const double t95 = in_H0 * t63;
    const double t96 = t94 + t95;
    const double t97 = pre[1] * t91;
    const double t98 = in_S1 * t66;
    const double t99 = t97 + t98;
    const double t100 = in_H1 * t63;
    const double t101 = t99 + t100;
    const double t102 = pre[2] * t91;
    const double t103 = in_S2 * t66;
    const double t104 = t102 + t103;
    const double t105 = in_H2 * t63;
    const double t106 = t104 + t105;
    const double t108 = t96 * pre[9];
    const double t109 = t101 * pre[9];
    const double t110 = t106 * pre[9];
    const double t111 = pre[1] * in_S2;
    const double t112 = pre[2] * in_S1;
    const double t113 = t111 - t112;
    const double t114 = pre[2] * in_S0;
    const double t115 = pre[0] * in_S2;
    const double t116 = t114 - t115;
    const double t117 = pre[0] * in_S1;
    const double t118 = pre[1] * in_S0;
    const double t119 = t117 - t118;
    const double t120 = pre[1] * in_H2;
    const double t121 = pre[2] * in_H1;
    const double t122 = t120 - t121;
    const double t123 = pre[2] * in_H0;
    const double t124 = pre[0] * in_H2;
    const double t125 = t123 - t124;
    const double t126 = pre[0] * in_H1;
    const double t127 = pre[1] * in_H0;
    const double t128 = t126 - t127;
    const double t129 = t66 * t113;
    const double t130 = -t129;
    const double t131 = t66 * t116;
    const double t132 = -t131;
    const double t133 = t66 * t119;
    const double t134 = -t133;
    const double t135 = t63 * t122;
    const double t136 = -t135;
    const double t137 = t63 * t125;
    const double t138 = -t137;
    const double t139 = t63 * t128;
    const double t140 = -t139;
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
    double d85[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d85[k] = d34[k] * pre[6];
    double d86[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d86[k] = d34[k] * t85 + t34 * d85[k];
    double d87[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d87[k] = d39[k] * pre[5];
    double d88[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d88[k] = d39[k] * t87 + t39 * d87[k];
    double d89[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d89[k] = d86[k] + d88[k];
    double d90[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d90[k] = dpre[8 * NT + k] * t89 + pre[8] * d89[k];
    double d91[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d91[k] = d82[k] + d90[k];
    double d92[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d92[k] = dpre[0 * NT + k] * t91 + pre[0] * d91[k];
    double d93[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d93[k] = din[3 * NT + k] * t66 + in_S0 * d66[k];
    double d94[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d94[k] = d92[k] + d93[k];
    double d95[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d95[k] = din[6 * NT + k] * t63 + in_H0 * d63[k];
    double d96[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d96[k] = d94[k] + d95[k];
    double d97[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d97[k] = dpre[1 * NT + k] * t91 + pre[1] * d91[k];
    double d98[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d98[k] = din[4 * NT + k] * t66 + in_S1 * d66[k];
    double d99[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d99[k] = d97[k] + d98[k];
    double d100[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d100[k] = din[7 * NT + k] * t63 + in_H1 * d63[k];
    double d101[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d101[k] = d99[k] + d100[k];
    double d102[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d102[k] = dpre[2 * NT + k] * t91 + pre[2] * d91[k];
    double d103[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d103[k] = din[5 * NT + k] * t66 + in_S2 * d66[k];
    double d104[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d104[k] = d102[k] + d103[k];
    double d105[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d105[k] = din[8 * NT + k] * t63 + in_H2 * d63[k];
    double d106[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d106[k] = d104[k] + d105[k];
    double d108[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d108[k] = d96[k] * pre[9];
    double d109[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d109[k] = d101[k] * pre[9];
    double d110[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d110[k] = d106[k] * pre[9];
    double d111[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d111[k] = dpre[1 * NT + k] * in_S2 + pre[1] * din[5 * NT + k];
    double d112[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d112[k] = dpre[2 * NT + k] * in_S1 + pre[2] * din[4 * NT + k];
    double d113[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d113[k] = d111[k] - d112[k];
    double d114[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d114[k] = dpre[2 * NT + k] * in_S0 + pre[2] * din[3 * NT + k];
    double d115[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d115[k] = dpre[0 * NT + k] * in_S2 + pre[0] * din[5 * NT + k];
    double d116[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d116[k] = d114[k] - d115[k];
    double d117[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d117[k] = dpre[0 * NT + k] * in_S1 + pre[0] * din[4 * NT + k];
    double d118[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d118[k] = dpre[1 * NT + k] * in_S0 + pre[1] * din[3 * NT + k];
    double d119[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d119[k] = d117[k] - d118[k];
    double d120[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d120[k] = dpre[1 * NT + k] * in_H2 + pre[1] * din[8 * NT + k];
    double d121[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d121[k] = dpre[2 * NT + k] * in_H1 + pre[2] * din[7 * NT + k];
    double d122[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d122[k] = d120[k] - d121[k];
    double d123[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d123[k] = dpre[2 * NT + k] * in_H0 + pre[2] * din[6 * NT + k];
    double d124[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d124[k] = dpre[0 * NT + k] * in_H2 + pre[0] * din[8 * NT + k];
    double d125[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d125[k] = d123[k] - d124[k];
    double d126[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d126[k] = dpre[0 * NT + k] * in_H1 + pre[0] * din[7 * NT + k];
    double d127[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d127[k] = dpre[1 * NT + k] * in_H0 + pre[1] * din[6 * NT + k];
    double d128[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d128[k] = d126[k] - d127[k];
    double d129[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d129[k] = d66[k] * t113 + t66 * d113[k];
    double d130[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d130[k] = -d129[k];
    double d131[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d131[k] = d66[k] * t116 + t66 * d116[k];
    double d132[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d132[k] = -d131[k];
    double d133[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d133[k] = d66[k] * t119 + t66 * d119[k];
    double d134[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d134[k] = -d133[k];
    double d135[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d135[k] = d63[k] * t122 + t63 * d122[k];
    double d136[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d136[k] = -d135[k];
    double d137[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d137[k] = d63[k] * t125 + t63 * d125[k];
    double d138[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d138[k] = -d137[k];
    double d139[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d139[k] = d63[k] * t128 + t63 * d128[k];
    double d140[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d140[k] = -d139[k];
    out[0] = t108;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[0 * NT + k] = d108[k];
    out[1] = t109;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[1 * NT + k] = d109[k];
    out[2] = t110;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[2 * NT + k] = d110[k];
    out[3] = t130;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[3 * NT + k] = d130[k];
    out[4] = t132;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[4 * NT + k] = d132[k];
    out[5] = t134;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[5 * NT + k] = d134[k];
    out[6] = t136;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[6 * NT + k] = d136[k];
    out[7] = t138;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[7 * NT + k] = d138[k];
    out[8] = t140;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[8 * NT + k] = d140[k];
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
    const double t51 = t49 / t50;
    const double t52 = t23 * t23;
    const double t53 = t33 * t48;
    const double t54 = -t48;
    const double t55 = kC2 * t52;
    const double t56 = t54 / t55;
    const double t58 = t51 * 3.0;
    const double t59 = 1.0 + t58;
    const double t61 = t51 + 2.0;
    const double t62 = 2.0 * t61;
    const double t63 = t53 * t62;
    const double t65 = t51 * 1.5;
    const double t66 = t48 / t55;
    const double t67 = 2.0 * t66;
    const double t68 = 2.0 - t51;
    const double t69 = t67 * t68;
    const double t71 = t51 * 29.0;
    const double t73 = t71 + 12.0;
    const double t75 = t73 * 0.75;
    const double t76 = t50 / t52;
    const double t77 = t75 * t76;
    const double t79 = t51 * 4.0;
    const double t80 = 3.0 - t79;
    const double t81 = t51 * t80;
    const double t83 = t51 * 1.875;
    const double t84 = 1.0 - t58;
    const double t85 = t83 * t84;
    const double t86 = t65 * t80;
    const double t88 = t51 * 0.5;
    const double t90 = 13.0 - t79;
    const double t91 = t88 * t90;
    const double t92 = t53 * t91;
    const double t94 = t51 * 25.0;
    const double t95 = 2.0 + t94;
    const double t96 = t51 * 2.0;
    const double t97 = t51 * t96;
    const double t98 = t95 + t97;
    const double t99 = t53 * t98;
    const double t101 = t56 * -0.5;
    const double t103 = t79 + 15.0;
    const double t104 = t51 * t103;
    const double t106 = t51 * 41.0;
    const double t107 = 4.0 + t106;
    const double t109 = t51 * 8.0;
    const double t110 = t51 * t109;
    const double t111 = t107 + t110;
    const double t112 = t53 * t111;
    const double t113 = 3.0 + t96;
    const double t114 = t58 * t113;
    const double t115 = t77 - t63;
    const double t116 = t59 - t92;
    const double t117 = t65 + t99;
    const double t118 = -t117;
    const double t119 = t101 * t112;
    const double t120 = t69 - t119;
    const double t121 = t101 * t104;
    const double t122 = t101 * t114;
    const double t123 = -t122;
    const double t156 = c_hm - c_m;
    const double t157 = c_moi * t156;
    const double t158 = t157 / c_m;
    const double t159 = t156 / c_hm;
    const double t182 = t34 * 6.0;
    const double t183 = t33 * t182;
    const double t184 = t35 * 6.0;
    const double t185 = t33 * t184;
    const double t186 = t36 * 6.0;
    const double t187 = t33 * t186;
    const double t250 = c_m * c_hm;
    const double t251 = c_m + c_hm;
    const double t252 = t250 / t251;
    const double t253 = c_m * 1.5;
    const double t254 = t253 / c_hm;
    const double t255 = 2.0 + t254;
    const double t256 = t252 * t255;
    const double t257 = c_hm * 1.5;
    const double t258 = t257 / c_m;
    const double t259 = 2.0 + t258;
    const double t260 = t252 * t259;
    pre[0] = in_x;
    pre[1] = in_y;
    pre[2] = in_z;
    pre[3] = t33;
    pre[4] = t81;
    pre[5] = t116;
    pre[6] = t86;
    pre[7] = t115;
    pre[8] = t85;
    pre[9] = t118;
    pre[10] = t56;
    pre[11] = t121;
    pre[12] = t120;
    pre[13] = t123;
    pre[14] = t34;
    pre[15] = t35;
    pre[16] = t36;
    pre[17] = t158;
    pre[18] = t159;
    pre[19] = t183;
    pre[20] = t185;
    pre[21] = t187;
    pre[22] = t256;
    pre[23] = t260;
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
    const double t124 = t42 * t42;
    const double t125 = t47 * pre[4];
    const double t126 = pre[5] + t125;
    const double t127 = pre[6] * t124;
    const double t128 = t126 - t127;
    const double t129 = t47 * t128;
    const double t130 = pre[7] + t129;
    const double t131 = pre[8] * t124;
    const double t132 = pre[9] + t131;
    const double t133 = t124 * t132;
    const double t134 = t130 + t133;
    const double t135 = pre[10] * t134;
    const double t136 = t47 * pre[11];
    const double t137 = pre[12] + t136;
    const double t138 = pre[13] * t124;
    const double t139 = t137 + t138;
    const double t140 = t42 * t139;
    const double t141 = pre[14] * t135;
    const double t142 = in_hv0 * t140;
    const double t143 = t141 + t142;
    const double t144 = pre[15] * t135;
    const double t145 = in_hv1 * t140;
    const double t146 = t144 + t145;
    const double t147 = pre[16] * t135;
    const double t148 = in_hv2 * t140;
    const double t149 = t147 + t148;
    const double t150 = in_H0 * c_hmoi;
    const double t151 = in_H1 * c_hmoi;
    const double t152 = in_H2 * c_hmoi;
    const double t153 = in_S0 * c_moi;
    const double t154 = in_S1 * c_moi;
    const double t155 = in_S2 * c_moi;
    const double t160 = in_S0 * pre[17];
    const double t161 = t150 * pre[18];
    const double t162 = t160 - t161;
    const double t163 = in_S1 * pre[17];
    const double t164 = t151 * pre[18];
    const double t165 = t163 - t164;
    const double t166 = in_S2 * pre[17];
    const double t167 = t152 * pre[18];
    const double t168 = t166 - t167;
    const double t169 = t150 + t153;
    const double t170 = t151 + t154;
    const double t171 = t152 + t155;
    const double t172 = pre[1] * in_hv2;
    const double t173 = pre[2] * in_hv1;
    const double t174 = t172 - t173;
    const double t175 = pre[2] * in_hv0;
    const double t176 = pre[0] * in_hv2;
    const double t177 = t175 - t176;
    const double t178 = pre[0] * in_hv1;
    const double t179 = pre[1] * in_hv0;
    const double t180 = t178 - t179;
    const double t188 = 2.0 * t169;
    const double t189 = t162 + t188;
    const double t190 = t174 * t189;
    const double t191 = pre[19] * t190;
    const double t192 = 2.0 * t170;
    const double t193 = t165 + t192;
    const double t194 = t177 * t193;
    const double t195 = pre[20] * t194;
    const double t196 = 2.0 * t171;
    const double t197 = t168 + t196;
    const double t198 = t180 * t197;
    const double t199 = pre[21] * t198;
    const double t200 = pre[14] * t42;
    const double t201 = t200 - in_hv0;
    const double t202 = pre[15] * t42;
    const double t203 = t202 - in_hv1;
    const double t204 = pre[16] * t42;
    const double t205 = t204 - in_hv2;
    const double t206 = t42 * 2.0;
    const double t208 = t201 * 7.0;
    const double t209 = pre[14] * t206;
    const double t210 = t208 + t209;
    const double t211 = t203 * 7.0;
    const double t212 = pre[15] * t206;
    const double t213 = t211 + t212;
    const double t214 = t205 * 7.0;
    const double t215 = pre[16] * t206;
    const double t216 = t214 + t215;
    const double t217 = t171 * t213;
    const double t218 = t170 * t216;
    const double t219 = t217 - t218;
    const double t220 = t169 * t216;
    const double t221 = t171 * t210;
    const double t222 = t220 - t221;
    const double t223 = t170 * t210;
    const double t224 = t169 * t213;
    const double t225 = t223 - t224;
    const double t226 = t168 * t203;
    const double t227 = t165 * t205;
    const double t228 = t226 - t227;
    const double t229 = t162 * t205;
    const double t230 = t168 * t201;
    const double t231 = t229 - t230;
    const double t232 = t165 * t201;
    const double t233 = t162 * t203;
    const double t234 = t232 - t233;
    const double t235 = t191 + t219;
    const double t236 = 3.0 * t228;
    const double t237 = t235 + t236;
    const double t238 = kFA * t237;
    const double t239 = t143 + t238;
    const double t240 = t195 + t222;
    const double t241 = 3.0 * t231;
    const double t242 = t240 + t241;
    const double t243 = kFA * t242;
    const double t244 = t146 + t243;
    const double t245 = t199 + t225;
    const double t246 = 3.0 * t234;
    const double t247 = t245 + t246;
    const double t248 = kFA * t247;
    const double t249 = t149 + t248;
    const double t261 = pre[14] * t153;
    const double t262 = pre[15] * t154;
    const double t263 = t261 + t262;
    const double t264 = pre[16] * t155;
    const double t265 = t263 + t264;
    const double t266 = 3.0 * t265;
    const double t267 = pre[14] * t150;
    const double t268 = pre[15] * t151;
    const double t269 = t267 + t268;
    const double t270 = pre[16] * t152;
    const double t271 = t269 + t270;
    const double t272 = 3.0 * t271;
    const double t273 = t174 * pre[22];
    const double t274 = t273 - t153;
    const double t275 = pre[14] * t266;
    const double t276 = t274 + t275;
    const double t277 = t177 * pre[22];
    const double t278 = t277 - t154;
    const double t279 = pre[15] * t266;
    const double t280 = t278 + t279;
    const double t281 = t180 * pre[22];
    const double t282 = t281 - t155;
    const double t283 = pre[16] * t266;
    const double t284 = t282 + t283;
    const double t285 = t174 * pre[23];
    const double t286 = t285 - t150;
    const double t287 = pre[14] * t272;
    const double t288 = t286 + t287;
    const double t289 = t177 * pre[23];
    const double t290 = t289 - t151;
    const double t291 = pre[15] * t272;
    const double t292 = t290 + t291;
    const double t293 = t180 * pre[23];
    const double t294 = t293 - t152;
    const double t295 = pre[16] * t272;
    const double t296 = t294 + t295;
    const double t297 = t152 * t280;
    const double t298 = t151 * t284;
    const double t299 = t297 - t298;
    const double t300 = t150 * t284;
    const double t301 = t152 * t276;
    const double t302 = t300 - t301;
    const double t303 = t151 * t276;
    const double t304 = t150 * t280;
    const double t305 = t303 - t304;
    const double t306 = t155 * t292;
    const double t307 = t154 * t296;
    const double t308 = t306 - t307;
    const double t309 = t153 * t296;
    const double t310 = t155 * t288;
    const double t311 = t309 - t310;
    const double t312 = t154 * t288;
    const double t313 = t153 * t292;
    const double t314 = t312 - t313;
    const double t315 = kFA * t299;
    const double t316 = kFA * t302;
    const double t317 = kFA * t305;
    const double t318 = kFA * t308;
    const double t319 = kFA * t311;
    const double t320 = kFA * t314;
    out[0] = t239;
    out[1] = t244;
    out[2] = t249;
    out[3] = t318;
    out[4] = t319;
    out[5] = t320;
    out[6] = t315;
    out[7] = t316;
    out[8] = t317;
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
    const double t124 = t42 * t42;
    const double t125 = t47 * pre[4];
    const double t126 = pre[5] + t125;
    const double t127 = pre[6] * t124;
    const double t128 = t126 - t127;
    const double t129 = t47 * t128;
    const double t130 = pre[7] + t129;
    const double t131 = pre[8] * t124;
    const double t132 = pre[9] + t131;
    const double t133 = t124 * t132;
    const double t134 = t130 + t133;
    const double t135 = pre[10] * t134;
    const double t136 = t47 * pre[11];
    const double t137 = pre[12] + t136;
    const double t138 = pre[13] * t124;
    const double t139 = t137 + t138;
    const double t140 = t42 * t139;
    const double t141 = pre[14] * t135;
    const double t142 = in_hv0 * t140;
    const double t143 = t141 + t142;
    const double t144 = pre[15] * t135;
    const double t145 = in_hv1 * t140;
    const double t146 = t144 + t145;
    const double t147 = pre[16] * t135;
    const double t148 = in_hv2 * t140;
    const double t149 = t147 + t148;
    const double t150 = in_H0 * c_hmoi;
    const double t151 = in_H1 * c_hmoi;
    const double t152 = in_H2 * c_hmoi;
    const double t153 = in_S0 * c_moi;
    const double t154 = in_S1 * c_moi;
    const double t155 = in_S2 * c_moi;
    const double t160 = in_S0 * pre[17];
    const double t161 = t150 * pre[18];
    const double t162 = t160 - t161;
    const double t163 = in_S1 * pre[17];
    const double t164 = t151 * pre[18];
    const double t165 = t163 - t164;
    const double t166 = in_S2 * pre[17];
    const double t167 = t152 * pre[18];
    const double t168 = t166 - t167;
    const double t169 = t150 + t153;
    const double t170 = t151 + t154;
    const double t171 = t152 + t155;
    const double t172 = pre[1] * in_hv2;
    const double t173 = pre[2] * in_hv1;
    const double t174 = t172 - t173;
    const double t175 = pre[2] * in_hv0;
    const double t176 = pre[0] * in_hv2;
    const double t177 = t175 - t176;
    const double t178 = pre[0] * in_hv1;
    const double t179 = pre[1] * in_hv0;
    const double t180 = t178 - t179;
    const double t188 = 2.0 * t169;
    const double t189 = t162 + t188;
    const double t190 = t174 * t189;
    const double t191 = pre[19] * t190;
    const double t192 = 2.0 * t170;
    const double t193 = t165 + t192;
    const double t194 = t177 * t193;
    const double t195 = pre[20] * t194;
    const double t196 = 2.0 * t171;
    const double t197 = t168 + t196;
    const double t198 = t180 * t197;
    const double t199 = pre[21] * t198;
    const double t200 = pre[14] * t42;
    const double t201 = t200 - in_hv0;
    const double t202 = pre[15] * t42;
    const double t203 = t202 - in_hv1;
    const double t204 = pre[16] * t42;
    const double t205 = t204 - in_hv2;
    const double t206 = t42 * 2.0;
    const double t208 = t201 * 7.0;
    const double t209 = pre[14] * t206;
    const double t210 = t208 + t209;
    const double t211 = t203 * 7.0;
    const double t212 = pre[15] * t206;
    const double t213 = t211 + t212;
    const double t214 = t205 * 7.0;
    const double t215 = pre[16] * t206;
    const double t216 = t214 + t215;
    const double t217 = t171 * t213;
    const double t218 = t170 * t216;
    const double t219 = t217 - t218;
    const double t220 = t169 * t216;
    const double t221 = t171 * t210;
    const double t222 = t220 - t221;
    const double t223 = t170 * t210;
    const double t224 = t169 * t213;
    const double t225 = t223 - t224;
    const double t226 = t168 * t203;
    const double t227 = t165 * t205;
    const double t228 = t226 - t227;
    const double t229 = t162 * t205;
    const double t230 = t168 * t201;
    const double t231 = t229 - t230;
    const double t232 = t165 * t201;
    const double t233 = t162 * t203;
    const double t234 = t232 - t233;
    const double t235 = t191 + t219;
    const double t236 = 3.0 * t228;
    const double t237 = t235 + t236;
    const double t238 = kFA * t237;
    const double t239 = t143 + t238;
    const double t240 = t195 + t222;
    const double t241 = 3.0 * t231;
    const double t242 = t240 + t241;
    const double t243 = kFA * t242;
    const double t244 = t146 + t243;
    const double t245 = t199 + t225;
    const double t246 = 3.0 * t234;
    const double t247 = t245 + t246;
    const double t248 = kFA * t247;
    const double t249 = t149 + t248;
    const double t261 = pre[14] * t153;
    const double t262 = pre[15] * t154;
    const double t263 = t261 + t262;
    const double t264 = pre[16] * t155;
    const double t265 = t263 + t264;
    const double t266 = 3.0 * t265;
    const double t267 = pre[14] * t150;
    const double t268 = pre[15] * t151;
    const double t269 = t267 + t268;
    const double t270 = pre[16] * t152;
    const double t271 = t269 + t270;
    const double t272 = 3.0 * t271;
    const double t273 = t174 * pre[22];
    const double t274 = t273 - t153;
    const double t275 = pre[14] * t266;
    const double t276 = t274 + t275;
    const double t277 = t177 * pre[22];
    const double t278 = t277 - t154;
    const double t279 = pre[15] * t266;
    const double t280 = t278 + t279;
    const double t281 = t180 * pre[22];
    const double t282 = t281 - t155;
    const double t283 = pre[16] * t266;
    const double t284 = t282 + t283;
    const double t285 = t174 * pre[23];
    const double t286 = t285 - t150;
    const double t287 = pre[14] * t272;
    const double t288 = t286 + t287;
    const double t289 = t177 * pre[23];
    const double t290 = t289 - t151;
    const double t291 = pre[15] * t272;
    const double t292 = t290 + t291;
    const double t293 = t180 * pre[23];
    const double t294 = t293 - t152;
    const double t295 = pre[16] * t272;
    const double t296 = t294 + t295;
    const double t297 = t152 * t280;
    const double t298 = t151 * t284;
    const double t299 = t297 - t298;
    const double t300 = t150 * t284;
    const double t301 = t152 * t276;
    const double t302 = t300 - t301;
    const double t303 = t151 * t276;
    const double t304 = t150 * t280;
    const double t305 = t303 - t304;
    const double t306 = t155 * t292;
    const double t307 = t154 * t296;
    const double t308 = t306 - t307;
    const double t309 = t153 * t296;
    const double t310 = t155 * t288;
    const double t311 = t309 - t310;
    const double t312 = t154 * t288;
    const double t313 = t153 * t292;
    const double t314 = t312 - t313;
    const double t315 = kFA * t299;
    const double t316 = kFA * t302;
    const double t317 = kFA * t305;
    const double t318 = kFA * t308;
    const double t319 = kFA * t311;
    const double t320 = kFA * t314;
    double b239 = bout[0];
    double b244 = bout[1];
    double b249 = bout[2];
    double b318 = bout[3];
    double b319 = bout[4];
    double b320 = bout[5];
    double b315 = bout[6];
    double b316 = bout[7];
    double b317 = bout[8];
    double b314 = b320 * kFA;
    double b311 = b319 * kFA;
    double b308 = b318 * kFA;
    double b305 = b317 * kFA;
    double b302 = b316 * kFA;
    double b299 = b315 * kFA;
    double b312 = b314;
    double b313 = -b314;
    double b153 = b313 * t292;
    double b292 = b313 * t153;
    double b154 = b312 * t288;
    double b288 = b312 * t154;
    double b309 = b311;
    double b310 = -b311;
    double b155 = b310 * t288;
    b288 += b310 * t155;
    b153 += b309 * t296;
    double b296 = b309 * t153;
    double b306 = b308;
    double b307 = -b308;
    b154 += b307 * t296;
    b296 += b307 * t154;
    b155 += b306 * t292;
    b292 += b306 * t155;
    double b303 = b305;
    double b304 = -b305;
    double b150 = b304 * t280;
    double b280 = b304 * t150;
    double b151 = b303 * t276;
    double b276 = b303 * t151;
    double b300 = b302;
    double b301 = -b302;
    double b152 = b301 * t276;
    b276 += b301 * t152;
    b150 += b300 * t284;
    double b284 = b300 * t150;
    double b297 = b299;
    double b298 = -b299;
    b151 += b298 * t284;
    b284 += b298 * t151;
    b152 += b297 * t280;
    b280 += b297 * t152;
    double b294 = b296;
    double b295 = b296;
    bpre[16] += b295 * t272;
    double b272 = b295 * pre[16];
    double b293 = b294;
    b152 += -b294;
    double b180 = b293 * pre[23];
    double b290 = b292;
    double b291 = b292;
    bpre[15] += b291 * t272;
    b272 += b291 * pre[15];
    double b289 = b290;
    b151 += -b290;
    double b177 = b289 * pre[23];
    double b286 = b288;
    double b287 = b288;
    bpre[14] += b287 * t272;
    b272 += b287 * pre[14];
    double b285 = b286;
    b150 += -b286;
    double b174 = b285 * pre[23];
    double b282 = b284;
    double b283 = b284;
    bpre[16] += b283 * t266;
    double b266 = b283 * pre[16];
    double b281 = b282;
    b155 += -b282;
    b180 += b281 * pre[22];
    double b278 = b280;
    double b279 = b280;
    bpre[15] += b279 * t266;
    b266 += b279 * pre[15];
    double b277 = b278;
    b154 += -b278;
    b177 += b277 * pre[22];
    double b274 = b276;
    double b275 = b276;
    bpre[14] += b275 * t266;
    b266 += b275 * pre[14];
    double b273 = b274;
    b153 += -b274;
    b174 += b273 * pre[22];
    double b271 = b272 * 3.0;
    double b269 = b271;
    double b270 = b271;
    bpre[16] += b270 * t152;
    b152 += b270 * pre[16];
    double b267 = b269;
    double b268 = b269;
    bpre[15] += b268 * t151;
    b151 += b268 * pre[15];
    bpre[14] += b267 * t150;
    b150 += b267 * pre[14];
    double b265 = b266 * 3.0;
    double b263 = b265;
    double b264 = b265;
    bpre[16] += b264 * t155;
    b155 += b264 * pre[16];
    double b261 = b263;
    double b262 = b263;
    bpre[15] += b262 * t154;
    b154 += b262 * pre[15];
    bpre[14] += b261 * t153;
    b153 += b261 * pre[14];
    double b149 = b249;
    double b248 = b249;
    double b247 = b248 * kFA;
    double b245 = b247;
    double b246 = b247;
    double b234 = b246 * 3.0;
    double b199 = b245;
    double b225 = b245;
    double b146 = b244;
    double b243 = b244;
    double b242 = b243 * kFA;
    double b240 = b242;
    double b241 = b242;
    double b231 = b241 * 3.0;
    double b195 = b240;
    double b222 = b240;
    double b143 = b239;
    double b238 = b239;
    double b237 = b238 * kFA;
    double b235 = b237;
    double b236 = b237;
    double b228 = b236 * 3.0;
    double b191 = b235;
    double b219 = b235;
    double b232 = b234;
    double b233 = -b234;
    double b162 = b233 * t203;
    double b203 = b233 * t162;
    double b165 = b232 * t201;
    double b201 = b232 * t165;
    double b229 = b231;
    double b230 = -b231;
    double b168 = b230 * t201;
    b201 += b230 * t168;
    b162 += b229 * t205;
    double b205 = b229 * t162;
    double b226 = b228;
    double b227 = -b228;
    b165 += b227 * t205;
    b205 += b227 * t165;
    b168 += b226 * t203;
    b203 += b226 * t168;
    double b223 = b225;
    double b224 = -b225;
    double b169 = b224 * t213;
    double b213 = b224 * t169;
    double b170 = b223 * t210;
    double b210 = b223 * t170;
    double b220 = b222;
    double b221 = -b222;
    double b171 = b221 * t210;
    b210 += b221 * t171;
    b169 += b220 * t216;
    double b216 = b220 * t169;
    double b217 = b219;
    double b218 = -b219;
    b170 += b218 * t216;
    b216 += b218 * t170;
    b171 += b217 * t213;
    b213 += b217 * t171;
    double b214 = b216;
    double b215 = b216;
    bpre[16] += b215 * t206;
    double b206 = b215 * pre[16];
    b205 += b214 * 7.0;
    double b211 = b213;
    double b212 = b213;
    bpre[15] += b212 * t206;
    b206 += b212 * pre[15];
    b203 += b211 * 7.0;
    double b208 = b210;
    double b209 = b210;
    bpre[14] += b209 * t206;
    b206 += b209 * pre[14];
    b201 += b208 * 7.0;
    double b42 = b206 * 2.0;
    double b204 = b205;
    double b_hv2 = -b205;
    bpre[16] += b204 * t42;
    b42 += b204 * pre[16];
    double b202 = b203;
    double b_hv1 = -b203;
    bpre[15] += b202 * t42;
    b42 += b202 * pre[15];
    double b200 = b201;
    double b_hv0 = -b201;
    bpre[14] += b200 * t42;
    b42 += b200 * pre[14];
    bpre[21] += b199 * t198;
    double b198 = b199 * pre[21];
    b180 += b198 * t197;
    double b197 = b198 * t180;
    b168 += b197;
    double b196 = b197;
    b171 += b196 * 2.0;
    bpre[20] += b195 * t194;
    double b194 = b195 * pre[20];
    b177 += b194 * t193;
    double b193 = b194 * t177;
    b165 += b193;
    double b192 = b193;
    b170 += b192 * 2.0;
    bpre[19] += b191 * t190;
    double b190 = b191 * pre[19];
    b174 += b190 * t189;
    double b189 = b190 * t174;
    b162 += b189;
    double b188 = b189;
    b169 += b188 * 2.0;
    double b178 = b180;
    double b179 = -b180;
    bpre[1] += b179 * in_hv0;
    b_hv0 += b179 * pre[1];
    bpre[0] += b178 * in_hv1;
    b_hv1 += b178 * pre[0];
    double b175 = b177;
    double b176 = -b177;
    bpre[0] += b176 * in_hv2;
    b_hv2 += b176 * pre[0];
    bpre[2] += b175 * in_hv0;
    b_hv0 += b175 * pre[2];
    double b172 = b174;
    double b173 = -b174;
    bpre[2] += b173 * in_hv1;
    b_hv1 += b173 * pre[2];
    bpre[1] += b172 * in_hv2;
    b_hv2 += b172 * pre[1];
    b152 += b171;
    b155 += b171;
    b151 += b170;
    b154 += b170;
    b150 += b169;
    b153 += b169;
    double b166 = b168;
    double b167 = -b168;
    b152 += b167 * pre[18];
    double b_S2 = b166 * pre[17];
    double b163 = b165;
    double b164 = -b165;
    b151 += b164 * pre[18];
    double b_S1 = b163 * pre[17];
    double b160 = b162;
    double b161 = -b162;
    b150 += b161 * pre[18];
    double b_S0 = b160 * pre[17];
    b_S2 += b155 * c_moi;
    b_S1 += b154 * c_moi;
    b_S0 += b153 * c_moi;
    double b_H2 = b152 * c_hmoi;
    double b_H1 = b151 * c_hmoi;
    double b_H0 = b150 * c_hmoi;
    double b147 = b149;
    double b148 = b149;
    b_hv2 += b148 * t140;
    double b140 = b148 * in_hv2;
    bpre[16] += b147 * t135;
    double b135 = b147 * pre[16];
    double b144 = b146;
    double b145 = b146;
    b_hv1 += b145 * t140;
    b140 += b145 * in_hv1;
    bpre[15] += b144 * t135;
    b135 += b144 * pre[15];
    double b141 = b143;
    double b142 = b143;
    b_hv0 += b142 * t140;
    b140 += b142 * in_hv0;
    bpre[14] += b141 * t135;
    b135 += b141 * pre[14];
    b42 += b140 * t139;
    double b139 = b140 * t42;
    double b137 = b139;
    double b138 = b139;
    bpre[13] += b138 * t124;
    double b124 = b138 * pre[13];
    bpre[12] += b137;
    double b136 = b137;
    double b47 = b136 * pre[11];
    bpre[11] += b136 * t47;
    bpre[10] += b135 * t134;
    double b134 = b135 * pre[10];
    double b130 = b134;
    double b133 = b134;
    b124 += b133 * t132;
    double b132 = b133 * t124;
    bpre[9] += b132;
    double b131 = b132;
    b124 += b131 * pre[8];
    bpre[7] += b130;
    double b129 = b130;
    b47 += b129 * t128;
    double b128 = b129 * t47;
    double b126 = b128;
    double b127 = -b128;
    b124 += b127 * pre[6];
    bpre[5] += b126;
    double b125 = b126;
    b47 += b125 * pre[4];
    b42 += 2.0 * b124 * t42;
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
    const double t51 = t49 / t50;
    const double t52 = t23 * t23;
    const double t53 = t33 * t48;
    const double t54 = -t48;
    const double t55 = kC2 * t52;
    const double t56 = t54 / t55;
    const double t58 = t51 * 3.0;
    const double t59 = 1.0 + t58;
    const double t61 = t51 + 2.0;
    const double t62 = 2.0 * t61;
    const double t63 = t53 * t62;
    const double t65 = t51 * 1.5;
    const double t66 = t48 / t55;
    const double t67 = 2.0 * t66;
    const double t68 = 2.0 - t51;
    const double t69 = t67 * t68;
    const double t71 = t51 * 29.0;
    const double t73 = t71 + 12.0;
    const double t75 = t73 * 0.75;
    const double t76 = t50 / t52;
    const double t77 = t75 * t76;
    const double t79 = t51 * 4.0;
    const double t80 = 3.0 - t79;
    const double t81 = t51 * t80;
    const double t83 = t51 * 1.875;
    const double t84 = 1.0 - t58;
    const double t85 = t83 * t84;
    const double t86 = t65 * t80;
    const double t88 = t51 * 0.5;
    const double t90 = 13.0 - t79;
    const double t91 = t88 * t90;
    const double t92 = t53 * t91;
    const double t94 = t51 * 25.0;
    const double t95 = 2.0 + t94;
    const double t96 = t51 * 2.0;
    const double t97 = t51 * t96;
    const double t98 = t95 + t97;
    const double t99 = t53 * t98;
    const double t101 = t56 * -0.5;
    const double t103 = t79 + 15.0;
    const double t104 = t51 * t103;
    const double t106 = t51 * 41.0;
    const double t107 = 4.0 + t106;
    const double t109 = t51 * 8.0;
    const double t110 = t51 * t109;
    const double t111 = t107 + t110;
    const double t112 = t53 * t111;
    const double t113 = 3.0 + t96;
    const double t114 = t58 * t113;
    const double t115 = t77 - t63;
    const double t116 = t59 - t92;
    const double t117 = t65 + t99;
    const double t118 = -t117;
    const double t119 = t101 * t112;
    const double t120 = t69 - t119;
    const double t121 = t101 * t104;
    const double t122 = t101 * t114;
    const double t123 = -t122;
    const double t156 = c_hm - c_m;
    const double t157 = c_moi * t156;
    const double t158 = t157 / c_m;
    const double t159 = t156 / c_hm;
    const double t182 = t34 * 6.0;
    const double t183 = t33 * t182;
    const double t184 = t35 * 6.0;
    const double t185 = t33 * t184;
    const double t186 = t36 * 6.0;
    const double t187 = t33 * t186;
    const double t250 = c_m * c_hm;
    const double t251 = c_m + c_hm;
    const double t252 = t250 / t251;
    const double t253 = c_m * 1.5;
    const double t254 = t253 / c_hm;
    const double t255 = 2.0 + t254;
    const double t256 = t252 * t255;
    const double t257 = c_hm * 1.5;
    const double t258 = t257 / c_m;
    const double t259 = 2.0 + t258;
    const double t260 = t252 * t259;
    double b_x = bpre[0];
    double b_y = bpre[1];
    double b_z = bpre[2];
    double b33 = bpre[3];
    double b116 = bpre[5];
    double b115 = bpre[7];
    double b118 = bpre[9];
    double b56 = bpre[10];
    double b121 = bpre[11];
    double b120 = bpre[12];
    double b123 = bpre[13];
    double b34 = bpre[14];
    double b35 = bpre[15];
    double b36 = bpre[16];
    double b183 = bpre[19];
    double b185 = bpre[20];
    double b187 = bpre[21];
    b33 += b187 * t186;
    double b186 = b187 * t33;
    b36 += b186 * 6.0;
    b33 += b185 * t184;
    double b184 = b185 * t33;
    b35 += b184 * 6.0;
    b33 += b183 * t182;
    double b182 = b183 * t33;
    b34 += b182 * 6.0;
    double b122 = -b123;
    double b101 = b122 * t114;
    b101 += b121 * t104;
    double b69 = b120;
    double b119 = -b120;
    b101 += b119 * t112;
    double b112 = b119 * t101;
    double b117 = -b118;
    double b99 = b117;
    double b92 = -b116;
    double b77 = b115;
    double b63 = -b115;
    double b53 = b112 * t111;
    b56 += b101 * -0.5;
    b53 += b99 * t98;
    b53 += b92 * t91;
    double b76 = b77 * t75;
    double b52 = -b76 * t76 / t52;
    double b67 = b69 * t68;
    double b66 = b67 * 2.0;
    double b55 = -b66 * t66 / t55;
    b53 += b63 * t62;
    b55 += -b56 * t56 / t55;
    b52 += b55 * kC2;
    b33 += b53 * t48;
    double b23 = 2.0 * b52 * t23;
    b_z += b36 * t33;
    b33 += b36 * in_z;
    b_y += b35 * t33;
    b33 += b35 * in_y;
    b_x += b34 * t33;
    b33 += b34 * in_x;
    b23 += -b33 * t33 / t23;
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
    const double t51 = t49 / t50;
    const double t52 = t23 * t23;
    const double t53 = t33 * t48;
    const double t54 = -t48;
    const double t55 = kC2 * t52;
    const double t56 = t54 / t55;
    const double t58 = t51 * 3.0;
    const double t59 = 1.0 + t58;
    const double t61 = t51 + 2.0;
    const double t62 = 2.0 * t61;
    const double t63 = t53 * t62;
    const double t65 = t51 * 1.5;
    const double t66 = t48 / t55;
    const double t67 = 2.0 * t66;
    const double t68 = 2.0 - t51;
    const double t69 = t67 * t68;
    const double t71 = t51 * 29.0;
    const double t73 = t71 + 12.0;
    const double t75 = t73 * 0.75;
    const double t76 = t50 / t52;
    const double t77 = t75 * t76;
    const double t79 = t51 * 4.0;
    const double t80 = 3.0 - t79;
    const double t81 = t51 * t80;
    const double t83 = t51 * 1.875;
    const double t84 = 1.0 - t58;
    const double t85 = t83 * t84;
    const double t86 = t65 * t80;
    const double t88 = t51 * 0.5;
    const double t90 = 13.0 - t79;
    const double t91 = t88 * t90;
    const double t92 = t53 * t91;
    const double t94 = t51 * 25.0;
    const double t95 = 2.0 + t94;
    const double t96 = t51 * 2.0;
    const double t97 = t51 * t96;
    const double t98 = t95 + t97;
    const double t99 = t53 * t98;
    const double t101 = t56 * -0.5;
    const double t103 = t79 + 15.0;
    const double t104 = t51 * t103;
    const double t106 = t51 * 41.0;
    const double t107 = 4.0 + t106;
    const double t109 = t51 * 8.0;
    const double t110 = t51 * t109;
    const double t111 = t107 + t110;
    const double t112 = t53 * t111;
    const double t113 = 3.0 + t96;
    const double t114 = t58 * t113;
    const double t115 = t77 - t63;
    const double t116 = t59 - t92;
    const double t117 = t65 + t99;
    const double t118 = -t117;
    const double t119 = t101 * t112;
    const double t120 = t69 - t119;
    const double t121 = t101 * t104;
    const double t122 = t101 * t114;
    const double t123 = -t122;
    const double t156 = c_hm - c_m;
    const double t157 = c_moi * t156;
    const double t158 = t157 / c_m;
    const double t159 = t156 / c_hm;
    const double t182 = t34 * 6.0;
    const double t183 = t33 * t182;
    const double t184 = t35 * 6.0;
    const double t185 = t33 * t184;
    const double t186 = t36 * 6.0;
    const double t187 = t33 * t186;
    const double t250 = c_m * c_hm;
    const double t251 = c_m + c_hm;
    const double t252 = t250 / t251;
    const double t253 = c_m * 1.5;
    const double t254 = t253 / c_hm;
    const double t255 = 2.0 + t254;
    const double t256 = t252 * t255;
    const double t257 = c_hm * 1.5;
    const double t258 = t257 / c_m;
    const double t259 = 2.0 + t258;
    const double t260 = t252 * t259;
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
    for (int k = 0; k < NT; ++k) d33[k] = -t33 * d23[k] / t23;
    double d34[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d34[k] = din[0 * NT + k] * t33 + in_x * d33[k];
    double d35[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d35[k] = din[1 * NT + k] * t33 + in_y * d33[k];
    double d36[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d36[k] = din[2 * NT + k] * t33 + in_z * d33[k];
    double d52[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d52[k] = 2.0 * t23 * d23[k];
    double d53[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d53[k] = d33[k] * t48;
    double d55[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d55[k] = kC2 * d52[k];
    double d56[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d56[k] = -t56 * d55[k] / t55;
    double d63[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d63[k] = d53[k] * t62;
    double d66[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d66[k] = -t66 * d55[k] / t55;
    double d67[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d67[k] = 2.0 * d66[k];
    double d69[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d69[k] = d67[k] * t68;
    double d76[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d76[k] = -t76 * d52[k] / t52;
    double d77[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d77[k] = t75 * d76[k];
    double d92[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d92[k] = d53[k] * t91;
    double d99[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d99[k] = d53[k] * t98;
    double d101[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d101[k] = d56[k] * -0.5;
    double d112[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d112[k] = d53[k] * t111;
    double d115[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d115[k] = d77[k] - d63[k];
    double d116[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d116[k] = -d92[k];
    double d117[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d117[k] = d99[k];
    double d118[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d118[k] = -d117[k];
    double d119[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d119[k] = d101[k] * t112 + t101 * d112[k];
    double d120[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d120[k] = d69[k] - d119[k];
    double d121[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d121[k] = d101[k] * t104;
    double d122[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d122[k] = d101[k] * t114;
    double d123[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d123[k] = -d122[k];
    double d182[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d182[k] = d34[k] * 6.0;
    double d183[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d183[k] = d33[k] * t182 + t33 * d182[k];
    double d184[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d184[k] = d35[k] * 6.0;
    double d185[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d185[k] = d33[k] * t184 + t33 * d184[k];
    double d186[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d186[k] = d36[k] * 6.0;
    double d187[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d187[k] = d33[k] * t186 + t33 * d186[k];
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
    pre[4] = t81;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[4 * NT + k] = 0.0;
    pre[5] = t116;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[5 * NT + k] = d116[k];
    pre[6] = t86;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[6 * NT + k] = 0.0;
    pre[7] = t115;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[7 * NT + k] = d115[k];
    pre[8] = t85;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[8 * NT + k] = 0.0;
    pre[9] = t118;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[9 * NT + k] = d118[k];
    pre[10] = t56;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[10 * NT + k] = d56[k];
    pre[11] = t121;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[11 * NT + k] = d121[k];
    pre[12] = t120;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[12 * NT + k] = d120[k];
    pre[13] = t123;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[13 * NT + k] = d123[k];
    pre[14] = t34;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[14 * NT + k] = d34[k];
    pre[15] = t35;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[15 * NT + k] = d35[k];
    pre[16] = t36;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[16 * NT + k] = d36[k];
    pre[17] = t158;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[17 * NT + k] = 0.0;
    pre[18] = t159;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[18 * NT + k] = 0.0;
    pre[19] = t183;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[19 * NT + k] = d183[k];
    pre[20] = t185;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[20 * NT + k] = d185[k];
    pre[21] = t187;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[21 * NT + k] = d187[k];
    pre[22] = t256;
#pragma unroll
    for (int k = 0; k < NT; ++k) dpre[22 * NT + k] = 0.0;
    pre[23] = t260;
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
    const double t124 = t42 * t42;
    const double t125 = t47 * pre[4];
    const double t126 = pre[5] + t125;
    const double t127 = pre[6] * t124;
    const double t128 = t126 - t127;
    const double t129 = t47 * t128;
    const double t130 = pre[7] + t129;
    const double t131 = pre[8] * t124;
    const double t132 = pre[9] + t131;
    const double t133 = t124 * t132;
    const double t134 = t130 + t133;
    const double t135 = pre[10] * t134;
    const double t136 = t47 * pre[11];
    const double t137 = pre[12] + t136;
    const double t138 = pre[13] * t124;
    const double t139 = t137 + t138;
    const double t140 = t42 * t139;
    const double t141 = pre[14] * t135;
    const double t142 = in_hv0 * t140;
    const double t143 = t141 + t142;
    const double t144 = pre[15] * t135;
    const double t145 = in_hv1 * t140;
    const double t146 = t144 + t145;
    const double t147 = pre[16] * t135;
    const double t148 = in_hv2 * t140;
    const double t149 = t147 + t148;
    const double t150 = in_H0 * c_hmoi;
    const double t151 = in_H1 * c_hmoi;
    const double t152 = in_H2 * c_hmoi;
    const double t153 = in_S0 * c_moi;
    const double t154 = in_S1 * c_moi;
    const double t155 = in_S2 * c_moi;
    const double t160 = in_S0 * pre[17];
    const double t161 = t150 * pre[18];
    const double t162 = t160 - t161;
    const double t163 = in_S1 * pre[17];
    const double t164 = t151 * pre[18];
    const double t165 = t163 - t164;
    const double t166 = in_S2 * pre[17];
    const double t167 = t152 * pre[18];
    const double t168 = t166 - t167;
    const double t169 = t150 + t153;
    const double t170 = t151 + t154;
    const double t171 = t152 + t155;
    const double t172 = pre[1] * in_hv2;
    const double t173 = pre[2] * in_hv1;
    const double t174 = t172 - t173;
    const double t175 = pre[2] * in_hv0;
    const double t176 = pre[0] * in_hv2;
    const double t177 = t175 - t176;
    const double t178 = pre[0] * in_hv1;
    const double t179 = pre[1] * in_hv0;
    const double t180 = t178 - t179;
    const double t188 = 2.0 * t169;
    const double t189 = t162 + t188;
    const double t190 = t174 * t189;
    const double t191 = pre[19] * t190;
    const double t192 = 2.0 * t170;
    const double t193 = t165 + t192;
    const double t194 = t177 * t193;
    const double t195 = pre[20] * t194;
    const double t196 = 2.0 * t171;
    const double t197 = t168 + t196;
    const double t198 = t180 * t197;
    const double t199 = pre[21] * t198;
    const double t200 = pre[14] * t42;
    const double t201 = t200 - in_hv0;
    const double t202 = pre[15] * t42;
    const double t203 = t202 - in_hv1;
    const double t204 = pre[16] * t42;
    const double t205 = t204 - in_hv2;
    const double t206 = t42 * 2.0;
    const double t208 = t201 * 7.0;
    const double t209 = pre[14] * t206;
    const double t210 = t208 + t209;
    const double t211 = t203 * 7.0;
    const double t212 = pre[15] * t206;
    const double t213 = t211 + t212;
    const double t214 = t205 * 7.0;
    const double t215 = pre[16] * t206;
    const double t216 = t214 + t215;
    const double t217 = t171 * t213;
    const double t218 = t170 * t216;
    const double t219 = t217 - t218;
    const double t220 = t169 * t216;
    const double t221 = t171 * t210;
    const double t222 = t220 - t221;
    const double t223 = t170 * t210;
    const double t224 = t169 * t213;
    const double t225 = t223 - t224;
    const double t226 = t168 * t203;
    const double t227 = t165 * t205;
    const double t228 = t226 - t227;
    const double t229 = t162 * t205;
    const double t230 = t168 * t201;
    const double t231 = t229 - t230;
    const double t232 = t165 * t201;
    const double t233 = t162 * t203;
    const double t234 = t232 - t233;
    const double t235 = t191 + t219;
    const double t236 = 3.0 * t228;
    const double t237 = t235 + t236;
    const double t238 = kFA * t237;
    const double t239 = t143 + t238;
    const double t240 = t195 + t222;
    const double t241 = 3.0 * t231;
    const double t242 = t240 + t241;
    const double t243 = kFA * t242;
    const double t244 = t146 + t243;
    const double t245 = t199 + t225;
    const double t246 = 3.0 * t234;
    const double t247 = t245 + t246;
    const double t248 = kFA * t247;
    const double t249 = t149 + t248;
    const double t261 = pre[14] * t153;
    const double t262 = pre[15] * t154;
    const double t263 = t261 + t262;
    const double t264 = pre[16] * t155;
    const double t265 = t263 + t264;
    const double t266 = 3.0 * t265;
    const double t267 = pre[14] * t150;
    const double t268 = pre[15] * t151;
    const double t269 = t267 + t268;
    const double t270 = pre[16] * t152;
    const double t271 = t269 + t270;
    const double t272 = 3.0 * t271;
    const double t273 = t174 * pre[22];
    const double t274 = t273 - t153;
    const double t275 = pre[14] * t266;
    const double t276 = t274 + t275;
    const double t277 = t177 * pre[22];
    const double t278 = t277 - t154;
    const double t279 = pre[15] * t266;
    const double t280 = t278 + t279;
    const double t281 = t180 * pre[22];
    const double t282 = t281 - t155;
    const double t283 = pre[16] * t266;
    const double t284 = t282 + t283;
    const double t285 = t174 * pre[23];
    const double t286 = t285 - t150;
    const double t287 = pre[14] * t272;
    const double t288 = t286 + t287;
    const double t289 = t177 * pre[23];
    const double t290 = t289 - t151;
    const double t291 = pre[15] * t272;
    const double t292 = t290 + t291;
    const double t293 = t180 * pre[23];
    const double t294 = t293 - t152;
    const double t295 = pre[16] * t272;
    const double t296 = t294 + t295;
    const double t297 = t152 * t280;
    const double t298 = t151 * t284;
    const double t299 = t297 - t298;
    const double t300 = t150 * t284;
    const double t301 = t152 * t276;
    const double t302 = t300 - t301;
    const double t303 = t151 * t276;
    const double t304 = t150 * t280;
    const double t305 = t303 - t304;
    const double t306 = t155 * t292;
    const double t307 = t154 * t296;
    const double t308 = t306 - t307;
    const double t309 = t153 * t296;
    const double t310 = t155 * t288;
    const double t311 = t309 - t310;
    const double t312 = t154 * t288;
    const double t313 = t153 * t292;
    const double t314 = t312 - t313;
    const double t315 = kFA * t299;
    const double t316 = kFA * t302;
    const double t317 = kFA * t305;
    const double t318 = kFA * t308;
    const double t319 = kFA * t311;
    const double t320 = kFA * t314;
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
    double d124[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d124[k] = 2.0 * t42 * d42[k];
    double d125[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d125[k] = d47[k] * pre[4];
    double d126[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d126[k] = dpre[5 * NT + k] + d125[k];
    double d127[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d127[k] = pre[6] * d124[k];
    double d128[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d128[k] = d126[k] - d127[k];
    double d129[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d129[k] = d47[k] * t128 + t47 * d128[k];
    double d130[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d130[k] = dpre[7 * NT + k] + d129[k];
    double d131[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d131[k] = pre[8] * d124[k];
    double d132[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d132[k] = dpre[9 * NT + k] + d131[k];
    double d133[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d133[k] = d124[k] * t132 + t124 * d132[k];
    double d134[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d134[k] = d130[k] + d133[k];
    double d135[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d135[k] = dpre[10 * NT + k] * t134 + pre[10] * d134[k];
    double d136[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d136[k] = d47[k] * pre[11] + t47 * dpre[11 * NT + k];
    double d137[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d137[k] = dpre[12 * NT + k] + d136[k];
    double d138[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d138[k] = dpre[13 * NT + k] * t124 + pre[13] * d124[k];
    double d139[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d139[k] = d137[k] + d138[k];
    double d140[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d140[k] = d42[k] * t139 + t42 * d139[k];
    double d141[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d141[k] = dpre[14 * NT + k] * t135 + pre[14] * d135[k];
    double d142[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d142[k] = din[0 * NT + k] * t140 + in_hv0 * d140[k];
    double d143[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d143[k] = d141[k] + d142[k];
    double d144[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d144[k] = dpre[15 * NT + k] * t135 + pre[15] * d135[k];
    double d145[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d145[k] = din[1 * NT + k] * t140 + in_hv1 * d140[k];
    double d146[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d146[k] = d144[k] + d145[k];
    double d147[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d147[k] = dpre[16 * NT + k] * t135 + pre[16] * d135[k];
    double d148[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d148[k] = din[2 * NT + k] * t140 + in_hv2 * d140[k];
    double d149[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d149[k] = d147[k] + d148[k];
    double d150[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d150[k] = din[6 * NT + k] * c_hmoi;
    double d151[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d151[k] = din[7 * NT + k] * c_hmoi;
    double d152[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d152[k] = din[8 * NT + k] * c_hmoi;
    double d153[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d153[k] = din[3 * NT + k] * c_moi;
    double d154[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d154[k] = din[4 * NT + k] * c_moi;
    double d155[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d155[k] = din[5 * NT + k] * c_moi;
    double d160[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d160[k] = din[3 * NT + k] * pre[17];
    double d161[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d161[k] = d150[k] * pre[18];
    double d162[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d162[k] = d160[k] - d161[k];
    double d163[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d163[k] = din[4 * NT + k] * pre[17];
    double d164[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d164[k] = d151[k] * pre[18];
    double d165[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d165[k] = d163[k] - d164[k];
    double d166[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d166[k] = din[5 * NT + k] * pre[17];
    double d167[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d167[k] = d152[k] * pre[18];
    double d168[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d168[k] = d166[k] - d167[k];
    double d169[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d169[k] = d150[k] + d153[k];
    double d170[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d170[k] = d151[k] + d154[k];
    double d171[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d171[k] = d152[k] + d155[k];
    double d172[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d172[k] = dpre[1 * NT + k] * in_hv2 + pre[1] * din[2 * NT + k];
    double d173[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d173[k] = dpre[2 * NT + k] * in_hv1 + pre[2] * din[1 * NT + k];
    double d174[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d174[k] = d172[k] - d173[k];
    double d175[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d175[k] = dpre[2 * NT + k] * in_hv0 + pre[2] * din[0 * NT + k];
    double d176[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d176[k] = dpre[0 * NT + k] * in_hv2 + pre[0] * din[2 * NT + k];
    double d177[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d177[k] = d175[k] - d176[k];
    double d178[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d178[k] = dpre[0 * NT + k] * in_hv1 + pre[0] * din[1 * NT + k];
    double d179[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d179[k] = dpre[1 * NT + k] * in_hv0 + pre[1] * din[0 * NT + k];
    double d180[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d180[k] = d178[k] - d179[k];
    double d188[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d188[k] = 2.0 * d169[k];
    double d189[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d189[k] = d162[k] + d188[k];
    double d190[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d190[k] = d174[k] * t189 + t174 * d189[k];
    double d191[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d191[k] = dpre[19 * NT + k] * t190 + pre[19] * d190[k];
    double d192[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d192[k] = 2.0 * d170[k];
    double d193[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d193[k] = d165[k] + d192[k];
    double d194[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d194[k] = d177[k] * t193 + t177 * d193[k];
    double d195[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d195[k] = dpre[20 * NT + k] * t194 + pre[20] * d194[k];
    double d196[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d196[k] = 2.0 * d171[k];
    double d197[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d197[k] = d168[k] + d196[k];
    double d198[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d198[k] = d180[k] * t197 + t180 * d197[k];
    double d199[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d199[k] = dpre[21 * NT + k] * t198 + pre[21] * d198[k];
    double d200[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d200[k] = dpre[14 * NT + k] * t42 + pre[14] * d42[k];
    double d201[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d201[k] = d200[k] - din[0 * NT + k];
    double d202[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d202[k] = dpre[15 * NT + k] * t42 + pre[15] * d42[k];
    double d203[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d203[k] = d202[k] - din[1 * NT + k];
    double d204[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d204[k] = dpre[16 * NT + k] * t42 + pre[16] * d42[k];
    double d205[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d205[k] = d204[k] - din[2 * NT + k];
    double d206[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d206[k] = d42[k] * 2.0;
    double d208[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d208[k] = d201[k] * 7.0;
    double d209[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d209[k] = dpre[14 * NT + k] * t206 + pre[14] * d206[k];
    double d210[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d210[k] = d208[k] + d209[k];
    double d211[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d211[k] = d203[k] * 7.0;
    double d212[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d212[k] = dpre[15 * NT + k] * t206 + pre[15] * d206[k];
    double d213[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d213[k] = d211[k] + d212[k];
    double d214[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d214[k] = d205[k] * 7.0;
    double d215[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d215[k] = dpre[16 * NT + k] * t206 + pre[16] * d206[k];
    double d216[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d216[k] = d214[k] + d215[k];
    double d217[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d217[k] = d171[k] * t213 + t171 * d213[k];
    double d218[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d218[k] = d170[k] * t216 + t170 * d216[k];
    double d219[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d219[k] = d217[k] - d218[k];
    double d220[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d220[k] = d169[k] * t216 + t169 * d216[k];
    double d221[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d221[k] = d171[k] * t210 + t171 * d210[k];
    double d222[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d222[k] = d220[k] - d221[k];
    double d223[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d223[k] = d170[k] * t210 + t170 * d210[k];
    double d224[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d224[k] = d169[k] * t213 + t169 * d213[k];
    double d225[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d225[k] = d223[k] - d224[k];
    double d226[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d226[k] = d168[k] * t203 + t168 * d203[k];
    double d227[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d227[k] = d165[k] * t205 + t165 * d205[k];
    double d228[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d228[k] = d226[k] - d227[k];
    double d229[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d229[k] = d162[k] * t205 + t162 * d205[k];
    double d230[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d230[k] = d168[k] * t201 + t168 * d201[k];
    double d231[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d231[k] = d229[k] - d230[k];
    double d232[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d232[k] = d165[k] * t201 + t165 * d201[k];
    double d233[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d233[k] = d162[k] * t203 + t162 * d203[k];
    double d234[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d234[k] = d232[k] - d233[k];
    double d235[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d235[k] = d191[k] + d219[k];
    double d236[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d236[k] = 3.0 * d228[k];
    double d237[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d237[k] = d235[k] + d236[k];
    double d238[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d238[k] = kFA * d237[k];
    double d239[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d239[k] = d143[k] + d238[k];
    double d240[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d240[k] = d195[k] + d222[k];
    double d241[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d241[k] = 3.0 * d231[k];
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
    for (int k = 0; k < NT; ++k) d245[k] = d199[k] + d225[k];
    double d246[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d246[k] = 3.0 * d234[k];
    double d247[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d247[k] = d245[k] + d246[k];
    double d248[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d248[k] = kFA * d247[k];
    double d249[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d249[k] = d149[k] + d248[k];
    double d261[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d261[k] = dpre[14 * NT + k] * t153 + pre[14] * d153[k];
    double d262[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d262[k] = dpre[15 * NT + k] * t154 + pre[15] * d154[k];
    double d263[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d263[k] = d261[k] + d262[k];
    double d264[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d264[k] = dpre[16 * NT + k] * t155 + pre[16] * d155[k];
    double d265[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d265[k] = d263[k] + d264[k];
    double d266[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d266[k] = 3.0 * d265[k];
    double d267[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d267[k] = dpre[14 * NT + k] * t150 + pre[14] * d150[k];
    double d268[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d268[k] = dpre[15 * NT + k] * t151 + pre[15] * d151[k];
    double d269[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d269[k] = d267[k] + d268[k];
    double d270[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d270[k] = dpre[16 * NT + k] * t152 + pre[16] * d152[k];
    double d271[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d271[k] = d269[k] + d270[k];
    double d272[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d272[k] = 3.0 * d271[k];
    double d273[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d273[k] = d174[k] * pre[22];
    double d274[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d274[k] = d273[k] - d153[k];
    double d275[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d275[k] = dpre[14 * NT + k] * t266 + pre[14] * d266[k];
    double d276[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d276[k] = d274[k] + d275[k];
    double d277[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d277[k] = d177[k] * pre[22];
    double d278[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d278[k] = d277[k] - d154[k];
    double d279[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d279[k] = dpre[15 * NT + k] * t266 + pre[15] * d266[k];
    double d280[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d280[k] = d278[k] + d279[k];
    double d281[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d281[k] = d180[k] * pre[22];
    double d282[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d282[k] = d281[k] - d155[k];
    double d283[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d283[k] = dpre[16 * NT + k] * t266 + pre[16] * d266[k];
    double d284[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d284[k] = d282[k] + d283[k];
    double d285[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d285[k] = d174[k] * pre[23];
    double d286[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d286[k] = d285[k] - d150[k];
    double d287[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d287[k] = dpre[14 * NT + k] * t272 + pre[14] * d272[k];
    double d288[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d288[k] = d286[k] + d287[k];
    double d289[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d289[k] = d177[k] * pre[23];
    double d290[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d290[k] = d289[k] - d151[k];
    double d291[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d291[k] = dpre[15 * NT + k] * t272 + pre[15] * d272[k];
    double d292[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d292[k] = d290[k] + d291[k];
    double d293[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d293[k] = d180[k] * pre[23];
    double d294[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d294[k] = d293[k] - d152[k];
    double d295[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d295[k] = dpre[16 * NT + k] * t272 + pre[16] * d272[k];
    double d296[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d296[k] = d294[k] + d295[k];
    double d297[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d297[k] = d152[k] * t280 + t152 * d280[k];
    double d298[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d298[k] = d151[k] * t284 + t151 * d284[k];
    double d299[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d299[k] = d297[k] - d298[k];
    double d300[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d300[k] = d150[k] * t284 + t150 * d284[k];
    double d301[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d301[k] = d152[k] * t276 + t152 * d276[k];
    double d302[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d302[k] = d300[k] - d301[k];
    double d303[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d303[k] = d151[k] * t276 + t151 * d276[k];
    double d304[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d304[k] = d150[k] * t280 + t150 * d280[k];
    double d305[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d305[k] = d303[k] - d304[k];
    double d306[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d306[k] = d155[k] * t292 + t155 * d292[k];
    double d307[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d307[k] = d154[k] * t296 + t154 * d296[k];
    double d308[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d308[k] = d306[k] - d307[k];
    double d309[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d309[k] = d153[k] * t296 + t153 * d296[k];
    double d310[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d310[k] = d155[k] * t288 + t155 * d288[k];
    double d311[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d311[k] = d309[k] - d310[k];
    double d312[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d312[k] = d154[k] * t288 + t154 * d288[k];
    double d313[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d313[k] = d153[k] * t292 + t153 * d292[k];
    double d314[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d314[k] = d312[k] - d313[k];
    double d315[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d315[k] = kFA * d299[k];
    double d316[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d316[k] = kFA * d302[k];
    double d317[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d317[k] = kFA * d305[k];
    double d318[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d318[k] = kFA * d308[k];
    double d319[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d319[k] = kFA * d311[k];
    double d320[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) d320[k] = kFA * d314[k];
    out[0] = t239;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[0 * NT + k] = d239[k];
    out[1] = t244;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[1 * NT + k] = d244[k];
    out[2] = t249;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[2 * NT + k] = d249[k];
    out[3] = t318;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[3 * NT + k] = d318[k];
    out[4] = t319;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[4 * NT + k] = d319[k];
    out[5] = t320;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[5 * NT + k] = d320[k];
    out[6] = t315;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[6 * NT + k] = d315[k];
    out[7] = t316;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[7 * NT + k] = d316[k];
    out[8] = t317;
#pragma unroll
    for (int k = 0; k < NT; ++k) dout[8 * NT + k] = d317[k];
}

}  // namespace posi_adj
