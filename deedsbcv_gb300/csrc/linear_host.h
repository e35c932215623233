// Host half of linearBCV: the least-trimmed-squares affine / rigid fit of
// src/QRsolve.h and the point selection of estimateAffine2 (src/affineLTS1.h:
// 160-236) from the per-node statistics the GPU computes.
#pragma once
#include <vector>

namespace deeds {

// Fewest points a fit accepts: below this the trimmed half of affineRobust has
// fewer than four points for four unknowns per row.
constexpr int kMinFitPoints = 8;

// qrsolve (src/QRsolve.h:18-84): least squares of A (len x 4, column c at
// A + c*len) against nrhs right-hand sides (column j at b + j*len) by classical
// Gram-Schmidt; solution j at X + 4j.
void lin_qrsolve(float* X, const float* A, const float* b, int len, int nrhs);

// affineRobust (src/QRsolve.h:258-296): points in column layout (y | x | z | 1),
// len points each; RT in the deeds matrix layout.  Does nothing for len <
// kMinFitPoints.
void lin_affine_robust(float* RT, const float* p1, const float* p2, int len, bool rigid);

// The host part of estimateAffine2 (src/affineLTS1.h:160-236): per node the
// (masked) minimum and its label of both smoothed cost volumes -> X = fit *
// Xprev.  minval/minind hold sz1 entries for the first volume followed by sz1
// for the second.  Returns the number of points used; *allcount receives the
// number of unmasked entries and *quantile the selection quantile.  With fewer
// than kMinFitPoints selected points X is not written.
int lin_estimate_from_stats(float* X, const float* Xprev, const float* minval, const int* minind, int m1, int n1,
                            int o1, int g, float q, int hw, bool rigid, int* allcount, float* quantile);

// X = A * B for 4x4 matrices (matmult, src/affineLTS1.h:1-12).
void lin_matmult(const float* A, const float* B, float* X);

}  // namespace deeds
