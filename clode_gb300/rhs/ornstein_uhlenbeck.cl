/* Ornstein-Uhlenbeck process dx = theta (mu - x) dt + sigma dW.
 * Parameters (theta, mu, sigma); one Wiener process. Under the stochastic
 * Euler stepper w[0] is N(0,1)/sqrt(dt), so dt*dx is the Euler-Maruyama step. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    dx_[0] = p_[0] * (p_[1] - x_[0]) + p_[2] * w_[0];
}
