// Host build of the adjoint building blocks, for the CPU tests of
// tests/test_adjoint_blocks.py (finite-difference checks of every VJP).
#include "../../posidonius_gb300/csrc/adjoint_effects.cuh"

using namespace posi_adj;

extern "C" {

void h_stumpff6(double z, double* c) { stumpff6(z, c); }

// in: r[3], v[3]; out: r1[3], v1[3]; returns X (NaN when not converged)
double h_kepler_fwd(double mu, double dt, const double* r, const double* v, double* r1, double* v1) {
    KeplerScalars s = kepler_scalars(mu, r, v);
    bool ok = false;
    double X = kepler_solve(s, dt, &ok);
    if (!ok) return NAN;
    kepler_apply(mu, dt, r, v, s, X, r1, v1);
    return X;
}

void h_kepler_vjp(double mu, double dt, const double* r, const double* v, double X, const double* lr1,
                  const double* lv1, double* lr0, double* lv0) {
    kepler_vjp(mu, dt, r, v, X, lr1, lv1, lr0, lv0);
}

// in: 22 inputs (x y z hv S H P Q sig_p sig_h k2_p k2_h); c: m hm R hR k2f hk2f mg hmg moi hmoi
#define ITER_ARGS(in) in[3], in[4], in[5], in[6], in[7], in[8], in[9], in[10], in[11], in[12], in[13], in[14], \
                      in[15], in[16], in[17]

void h_effects_fwd(int which, const double* in, const double* c, double* out) {
    const double m = c[0], hm = c[1], R = c[2], hR = c[3], k2f = c[4], hk2f = c[5], mg = c[6], hmg = c[7];
    const double moi = c[8], hmoi = c[9];
    double pre[64];
    if (which == 0) {
        adj_tides_pre(in[0], in[1], in[2], in[18], in[19], in[20], in[21], R, hR, hm, m, pre);
        adj_tides_iter(pre, ITER_ARGS(in), R, hR, hm, m, out);
    } else if (which == 1) {
        adj_flat_pre(in[0], in[1], in[2], R, hR, hk2f, hm, k2f, m, pre);
        adj_flat_iter(pre, ITER_ARGS(in), R, hR, hk2f, hm, k2f, m, out);
    } else {
        adj_gr_pre(in[0], in[1], in[2], hm, hmg, hmoi, m, mg, moi, pre);
        adj_gr_iter(pre, ITER_ARGS(in), hm, hmg, hmoi, m, mg, moi, out);
    }
}

// bin[22] += adjoints in the input order of h_effects_fwd
void h_effects_vjp(int which, const double* in, const double* c, const double* bout, double* bin) {
    const double m = c[0], hm = c[1], R = c[2], hR = c[3], k2f = c[4], hk2f = c[5], mg = c[6], hmg = c[7];
    const double moi = c[8], hmoi = c[9];
    double pre[64], bpre[64], bit[15], bp[7];
    for (int k = 0; k < 64; ++k) bpre[k] = 0.;
    for (int k = 0; k < 15; ++k) bit[k] = 0.;
    for (int k = 0; k < 7; ++k) bp[k] = 0.;
    if (which == 0) {
        adj_tides_pre(in[0], in[1], in[2], in[18], in[19], in[20], in[21], R, hR, hm, m, pre);
        adj_tides_iter_vjp(pre, ITER_ARGS(in), R, hR, hm, m, bout, bit, bpre);
        adj_tides_pre_vjp(in[0], in[1], in[2], in[18], in[19], in[20], in[21], R, hR, hm, m, bpre, bp);
    } else if (which == 1) {
        adj_flat_pre(in[0], in[1], in[2], R, hR, hk2f, hm, k2f, m, pre);
        adj_flat_iter_vjp(pre, ITER_ARGS(in), R, hR, hk2f, hm, k2f, m, bout, bit, bpre);
        adj_flat_pre_vjp(in[0], in[1], in[2], R, hR, hk2f, hm, k2f, m, bpre, bp);
    } else {
        adj_gr_pre(in[0], in[1], in[2], hm, hmg, hmoi, m, mg, moi, pre);
        adj_gr_iter_vjp(pre, ITER_ARGS(in), hm, hmg, hmoi, m, mg, moi, bout, bit, bpre);
        adj_gr_pre_vjp(in[0], in[1], in[2], hm, hmg, hmoi, m, mg, moi, bpre, bp);
    }
    for (int k = 0; k < 3; ++k) bin[k] += bp[k];
    for (int k = 0; k < 15; ++k) bin[3 + k] += bit[k];
    for (int k = 0; k < 4; ++k) bin[18 + k] += bp[3 + k];
}

void h_kepler_jvp(double mu, double dt, const double* r, const double* v, double X, const double* dr,
                  const double* dv, double* dr1, double* dv1) {
    kepler_jvp(mu, dt, r, v, X, dr, dv, dr1, dv1);
}

// tangent of the 9 outputs along din (22 inputs, one direction)
void h_effects_jvp(int which, const double* in, const double* c, const double* din, double* dout) {
    const double m = c[0], hm = c[1], R = c[2], hR = c[3], k2f = c[4], hk2f = c[5], mg = c[6], hmg = c[7];
    const double moi = c[8], hmoi = c[9];
    double pre[64], dpre[64], out[9], dpin[7], dit[15];
    for (int k = 0; k < 3; ++k) dpin[k] = din[k];
    for (int k = 0; k < 4; ++k) dpin[3 + k] = din[18 + k];
    for (int k = 0; k < 15; ++k) dit[k] = din[3 + k];
    if (which == 0) {
        adj_tides_pre_jvp<1>(in[0], in[1], in[2], in[18], in[19], in[20], in[21], R, hR, hm, m, dpin, pre, dpre);
        adj_tides_iter_jvp<1>(pre, dpre, ITER_ARGS(in), R, hR, hm, m, dit, out, dout);
    } else if (which == 1) {
        adj_flat_pre_jvp<1>(in[0], in[1], in[2], R, hR, hk2f, hm, k2f, m, dpin, pre, dpre);
        adj_flat_iter_jvp<1>(pre, dpre, ITER_ARGS(in), R, hR, hk2f, hm, k2f, m, dit, out, dout);
    } else {
        adj_gr_pre_jvp<1>(in[0], in[1], in[2], hm, hmg, hmoi, m, mg, moi, dpin, pre, dpre);
        adj_gr_iter_jvp<1>(pre, dpre, ITER_ARGS(in), hm, hmg, hmoi, m, mg, moi, dit, out, dout);
    }
}

}  // extern "C"
