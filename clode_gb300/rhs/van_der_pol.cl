/* Van der Pol oscillator: x' = y, y' = mu (1 - x^2) y - x.
 * State (x, y); parameter mu. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    realtype mu = p_[0];
    realtype x = x_[0];
    realtype y = x_[1];
    dx_[0] = y;
    dx_[1] = mu * (1 - x * x) * y - x;
}
