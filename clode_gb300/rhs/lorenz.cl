/* Lorenz system. State (x, y, z); parameters (rho, sigma, beta), in that order.
 * aux[0] records dx/dt. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    realtype x = x_[0], y = x_[1], z = x_[2];
    realtype rho = p_[0], sigma = p_[1], beta = p_[2];
    realtype fx = sigma * (y - x);
    dx_[0] = fx;
    dx_[1] = rho * x - y - x * z;
    dx_[2] = x * y - beta * z;
    aux_[0] = fx;
}
