// adjoint_record.h -- layout of the per-step record of the adjoint.
//
// For every step and body, the values the step's vector-Jacobian product
// needs, stored field-major over the bodies of the ensemble
// (record[(step * POSI_REC_COUNT + field) * stride + body]).  Written by the
// record pass (the FAST forward kernel, or the adjoint's own forward for an
// EXACT batch), read by the reverse sweep.  Midpoint blocks: the iteration
// count, then per iteration the velocity, spin angular momentum and previous
// spin the additional effects were evaluated with.
#pragma once

namespace posi_rec {
constexpr int kMidMax = 10;  // implicit-midpoint iterations at most
enum {
    SV_TRIG = 0,   // the step opened with a spin refresh (historic snapshot)
    SV_R0 = 1,     // inertial position at the step start
    SV_RJA = 4,    // Jacobi position / velocity before the first Kepler drift
    SV_VJA = 7,
    SV_X1 = 10,    // universal anomaly of the first drift
    SV_RJB = 11,   // Jacobi position / velocity after it
    SV_VJB = 14,
    SV_RG = 17,    // inertial position at the gravity evaluation
    SV_VJC = 20,   // Jacobi velocity after the interaction kick
    SV_X2 = 23,    // universal anomaly of the second drift
    SV_R2 = 24,    // inertial position at the second half kick
    SV_H1 = 27,    // first half kick
    SV_MID = 1 + 9 * kMidMax,
    SV_H2 = SV_H1 + SV_MID,
    SV_COUNT = SV_H2 + SV_MID
};
}  // namespace posi_rec
