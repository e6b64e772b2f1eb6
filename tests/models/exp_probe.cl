/* aux_[0] = exp(x): the exp builtin on each member's state (dx = 0). */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    aux_[0] = exp(x_[0]);
    dx_[0] = ZERO;
}
