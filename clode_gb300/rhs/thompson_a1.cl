/* Linear drag problem (ORNL report, Thompson problem A1):
 * y1' = y2, y2' = (w - k y2)/m; parameters (m, w, k, H); aux[0] = y1 - H.
 * Exact solution from rest: y1 = 4 (t + exp(-8t)/8 - 1/8), y2 = 4 (1 - exp(-8t))
 * for m = 1/4, w = 8, k = 2. */
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    dx_[0] = x_[1];
    dx_[1] = (p_[1] - p_[2] * x_[1]) / p_[0];
    aux_[0] = x_[0] - p_[3];
}
