/* A model in the form clODE's XPP translator writes (clode/xpp_parser.py:73-167):
 * decimal literals carry an `f` suffix, and parameters and auxiliaries are
 * named locals.  FitzHugh-Nagumo with a Heaviside drive. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[], realtype dx_[], realtype aux_[],
            const realtype w_[])
{
    realtype a = p_[0];
    realtype b = p_[1];
    realtype v = x_[0];
    realtype r = x_[1];
    realtype drive = 0.5f * heaviside(t - 10.0f);
    dx_[0] = v - v * v * v / 3.0f - r + drive;
    dx_[1] = 0.08f * (v + a - b * r);
    aux_[0] = exp(-0.1f * t) * drive;
}
