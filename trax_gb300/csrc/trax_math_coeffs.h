// Generated by fit_math_coeffs.py -- polynomial kernels of trax_math.h.
// f(t) = t + t^3 * P(t^2),  P(u) = C0 + C1 u + ... (Horner, float32).
// Weighted least squares + Lawson iterations on Chebyshev nodes; see the
// script for the fitting method.  Max relative error of the float32 kernel
// over its interval is given in units of 2^-24 beside each table.
#pragma once

// atan: t in [0, 0.414213562], max rel err 1.05 x 2^-24
#define TRAX_ATAN_NCOEF 7
#define TRAX_ATAN_COEFS { -3.333333433e-01f, 1.999999434e-01f, -1.428542435e-01f, 1.110400409e-01f, -8.996845037e-02f, 6.991240382e-02f, -3.792475536e-02f }

// asin: t in [0, 0.5], max rel err 1.07 x 2^-24
#define TRAX_ASIN_NCOEF 7
#define TRAX_ASIN_COEFS { 1.666666716e-01f, 7.499948889e-02f, 4.465997219e-02f, 3.011252545e-02f, 2.460470796e-02f, 7.509485818e-03f, 3.464631364e-02f }

// atanh: t in [0, 0.171572875], max rel err 1.00 x 2^-24
#define TRAX_ATANH_NCOEF 5
#define TRAX_ATANH_COEFS { 3.333333433e-01f, 1.999999732e-01f, 1.428605467e-01f, 1.108811945e-01f, 9.791719168e-02f }

// asinh: t in [0, 1], max rel err 1.10 x 2^-24
#define TRAX_ASINH_NCOEF 13
#define TRAX_ASINH_COEFS { -1.666666716e-01f, 7.499999553e-02f, -4.464269429e-02f, 3.037952445e-02f, -2.235094644e-02f, 1.723148860e-02f, -1.348629035e-02f, 1.019633468e-02f, -6.920428015e-03f, 3.852281952e-03f, -1.582941040e-03f, 4.152705369e-04f, -5.134236926e-05f }
