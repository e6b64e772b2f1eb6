/* Lactotroph model (see lactotroph.cl) with an additive white-noise current
 * sig * w[0]; parameters (gcal, gsk, gbk, sig), one Wiener process. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    realtype v = x_[0], n = x_[1], f = x_[2], c = x_[3];
    realtype csq = c * c;
    realtype kdrive = v - RCONST(-75.0);
    realtype m_inf = RCONST(1.0) / (RCONST(1.0) + exp((RCONST(-20.0) - v) / RCONST(12.0)));
    realtype n_inf = RCONST(1.0) / (RCONST(1.0) + exp((RCONST(-5.0) - v) / RCONST(10.0)));
    realtype i_ca = p_[0] * m_inf * (v - RCONST(60.0));
    realtype i_sk = p_[1] * csq / (csq + RCONST(0.40) * RCONST(0.40)) * kdrive;
    realtype i_bk = p_[2] * f * kdrive;
    realtype i_k = RCONST(2.0) * n * kdrive;
    realtype i_l = RCONST(0.050) * (v - RCONST(-50.0));
    realtype i_noise = p_[3] * w_[0];
    realtype i_tot = i_ca + i_sk + i_bk + i_k + i_l + i_noise;
    dx_[0] = -i_tot / RCONST(10.0);
    dx_[1] = (n_inf - n) / RCONST(30.0);
    dx_[2] = (RCONST(1.0) / (RCONST(1.0) + exp((RCONST(-20.0) - v) / RCONST(2.0))) - f) / RCONST(8.0);
    dx_[3] = -RCONST(0.010) * (RCONST(0.00150) * i_ca + RCONST(0.20) * c);
    aux_[0] = i_ca;
}
