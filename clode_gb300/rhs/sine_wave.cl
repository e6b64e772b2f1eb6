/* x' = cos(k t): x(t) = sin(k t)/k from x(0) = 0. Parameter k.
 * aux = (x + 1, 1, -2): constant and shifted outputs for observer checks. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    dx_[0] = cos(t * p_[0]);
    aux_[0] = x_[0] + RCONST(1.0);
    aux_[1] = RCONST(1.0);
    aux_[2] = RCONST(-2.0);
}
