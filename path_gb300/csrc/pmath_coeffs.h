// Generated by gen_pmath.py: polynomial coefficients for pmath.h.
// Each array lists coefficients from the constant term upwards.
#pragma once

#define PM_SIN_DEGREE 4
#define PM_SIN_COEFFS {-1.666666716e-01f, 8.333333768e-03f, -1.984126429e-04f, 2.755533842e-06f, -2.476041594e-08f}

#define PM_COS_DEGREE 4
#define PM_COS_COEFFS {4.166666791e-02f, -1.388888923e-03f, 2.480158037e-05f, -2.755542425e-07f, 2.063925919e-09f}

#define PM_ASIN_DEGREE 6
#define PM_ASIN_COEFFS {1.666666716e-01f, 7.499948889e-02f, 4.465997219e-02f, 3.011252731e-02f, 2.460470051e-02f, 7.509509567e-03f, 3.464628384e-02f}

