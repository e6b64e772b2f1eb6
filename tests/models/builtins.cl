/* Every OpenCL math builtin that clODE's Python converter can emit
 * (clode/function_converter.py:54-124), each evaluated on the state scaled
 * by t, with the arguments of clODE's own builtin test
 * (test/test_opencl_builtins.py:81-138).  x = (0.3, 1.5, 2.5) stays constant
 * (dx = 0); p = (2.8, 4.55) supplies the integer arguments.  aux_[k] holds
 * builtin k. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    const int p0 = (int)p_[0];
    const int p1 = (int)p_[1];
    const realtype x0 = x_[0] * t;
    const realtype x1 = x_[1] * t;
    realtype c;
    aux_[0] = acos(x0);
    aux_[1] = acosh(x0 + RCONST(1.0));
    aux_[2] = acospi(x0);
    aux_[3] = asin(x0);
    aux_[4] = asinh(x0 + RCONST(1.0));
    aux_[5] = asinpi(x0);
    aux_[6] = atan(x0);
    aux_[7] = atan2(x0, x1);
    aux_[8] = atan2pi(x0, x1);
    aux_[9] = atanh(x0 / RCONST(100.0));
    aux_[10] = atanpi(x0);
    aux_[11] = cbrt(x0);
    aux_[12] = ceil(x0);
    aux_[13] = copysign(x0, x1);
    aux_[14] = cos(x0);
    aux_[15] = cosh(x0);
    aux_[16] = cospi(x0);
    aux_[17] = erf(x0);
    aux_[18] = erfc(x0);
    aux_[19] = exp(x0);
    aux_[20] = exp2(x0);
    aux_[21] = exp10(x0);
    aux_[22] = expm1(x0);
    aux_[23] = fabs(x0);
    aux_[24] = fdim(x0, x1);
    aux_[25] = floor(x1);
    aux_[26] = fmax(x0, x1);
    aux_[27] = fmod(x0, x1 + RCONST(1.0));
    aux_[28] = heaviside(t - RCONST(0.5));
    aux_[29] = tgamma(x0 + RCONST(1.0));
    aux_[30] = hypot(x0, x1);
    aux_[31] = (realtype)ilogb(x0 + RCONST(1.0));
    aux_[32] = ldexp(x0, (int)x1);
    aux_[33] = lgamma(x0 + RCONST(1.0));
    aux_[34] = log(x0 + RCONST(1.0));
    aux_[35] = log1p(x0 + RCONST(1.0));
    aux_[36] = log2(x0 + RCONST(1.0));
    aux_[37] = log10(x0 + RCONST(1.0));
    aux_[38] = fmin(x0, x1);
    aux_[39] = sincos(x0, &c) + c;
    aux_[40] = sinh(x0) - tanh(x0);
    aux_[41] = nextafter(x0, x1);
    aux_[42] = pow(x0, x1);
    aux_[43] = pown(x0, p0);
    aux_[44] = powr(x0 + RCONST(0.5), x1 + RCONST(0.2));
    aux_[45] = remainder(x0, x1 + RCONST(1.0));
    aux_[46] = rint(x0);
    aux_[47] = rootn(x0, p1);
    aux_[48] = rsqrt(x0 + RCONST(1.0));
    aux_[49] = sin(x0);
    aux_[50] = sinh(x0);
    aux_[51] = sinpi(x0);
    aux_[52] = sqrt(x0);
    aux_[53] = tan(x0);
    aux_[54] = tanh(x0);
    aux_[55] = tanpi(x0);
    aux_[56] = trunc(x0);
    aux_[57] = round(x0 + RCONST(0.2));
    dx_[0] = ZERO;
    dx_[1] = ZERO;
    dx_[2] = ZERO;
}
