/*
 * D3Q19 BGK lattice-Boltzmann arithmetic shared by the oracle's two CPU
 * restatements (the reference-API cell in ref_driver.cpp and the plain C
 * oracle in lgd_oracle.c).  Test infrastructure only.
 *
 * Direction names and the incompressible BGK collision follow the
 * reference's LBM example (src/examples/latticeboltzmann/main.cpp:27-50 for
 * the names, :93-170 for the collision): rho and u are plain moments (u is
 * not divided by rho), dir_indep = rho/3 - u.u/2, and population i relaxes
 * towards 3 w_i (dir_indep + e_i.u + 1.5 (e_i.u)^2).
 *
 * Populations are pulled: f_i(x, t+1) = f*_i(x - e_i, t).  When x - e_i is
 * outside the fluid box the population is bounced back from the cell
 * itself, f*_{opp(i)}(x, t) + 6 w_i (e_i . u_wall), where u_wall is
 * (lid, 0, 0) for the lid (the wall beyond y = L-1) and 0 elsewhere.
 */
#ifndef LGD_ORACLE_LBM_D3Q19_H
#define LGD_ORACLE_LBM_D3Q19_H

enum {
    LGD_Q_C = 0, LGD_Q_N, LGD_Q_E, LGD_Q_W, LGD_Q_S, LGD_Q_T, LGD_Q_B,
    LGD_Q_NW, LGD_Q_SW, LGD_Q_NE, LGD_Q_SE,
    LGD_Q_TW, LGD_Q_BW, LGD_Q_TE, LGD_Q_BE,
    LGD_Q_TN, LGD_Q_BN, LGD_Q_TS, LGD_Q_BS
};

/* e_i = (x, y, z); N = +y, E = +x, T = +z */
static const int LGD_D3Q19_E[19][3] = {
    { 0,  0,  0},
    { 0,  1,  0}, { 1,  0,  0}, {-1,  0,  0}, { 0, -1,  0}, { 0,  0,  1}, { 0,  0, -1},
    {-1,  1,  0}, {-1, -1,  0}, { 1,  1,  0}, { 1, -1,  0},
    {-1,  0,  1}, {-1,  0, -1}, { 1,  0,  1}, { 1,  0, -1},
    { 0,  1,  1}, { 0,  1, -1}, { 0, -1,  1}, { 0, -1, -1}
};

static const int LGD_D3Q19_OPP[19] = {
    LGD_Q_C,
    LGD_Q_S, LGD_Q_W, LGD_Q_E, LGD_Q_N, LGD_Q_B, LGD_Q_T,
    LGD_Q_SE, LGD_Q_NE, LGD_Q_SW, LGD_Q_NW,
    LGD_Q_BE, LGD_Q_TE, LGD_Q_BW, LGD_Q_TW,
    LGD_Q_BS, LGD_Q_TS, LGD_Q_BN, LGD_Q_TN
};

static const double LGD_D3Q19_W[19] = {
    1.0 / 3.0,
    1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
    1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
    1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
    1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0
};

/* bounce-back of population i from the cell's own post-collision values */
static inline double lgd_d3q19_bounce(const double *self, int i, double lidVelocity)
{
    return self[LGD_D3Q19_OPP[i]] + 6.0 * LGD_D3Q19_W[i] * (LGD_D3Q19_E[i][0] * lidVelocity);
}

/* BGK collision of the pulled populations f into out */
static inline void lgd_d3q19_collide(const double *f, double omega, double *out)
{
    double rho = 0.0;
    int i;
    for (i = 0; i < 19; ++i) {
        rho += f[i];
    }
    const double ux =
        (f[LGD_Q_E] + f[LGD_Q_NE] + f[LGD_Q_SE] + f[LGD_Q_TE] + f[LGD_Q_BE]) -
        (f[LGD_Q_W] + f[LGD_Q_NW] + f[LGD_Q_SW] + f[LGD_Q_TW] + f[LGD_Q_BW]);
    const double uy =
        (f[LGD_Q_N] + f[LGD_Q_NW] + f[LGD_Q_NE] + f[LGD_Q_TN] + f[LGD_Q_BN]) -
        (f[LGD_Q_S] + f[LGD_Q_SW] + f[LGD_Q_SE] + f[LGD_Q_TS] + f[LGD_Q_BS]);
    const double uz =
        (f[LGD_Q_T] + f[LGD_Q_TW] + f[LGD_Q_TE] + f[LGD_Q_TN] + f[LGD_Q_TS]) -
        (f[LGD_Q_B] + f[LGD_Q_BW] + f[LGD_Q_BE] + f[LGD_Q_BN] + f[LGD_Q_BS]);
    const double usq = ux * ux + uy * uy + uz * uz;
    const double d = rho * (1.0 / 3.0) - 0.5 * usq;
    const double keep = 1.0 - omega;
    const double w1 = omega * (1.0 / 6.0);
    const double w2 = omega * (1.0 / 12.0);

    out[LGD_Q_C] = keep * f[LGD_Q_C] + omega * d;
    for (i = 1; i < 19; ++i) {
        const double eu = LGD_D3Q19_E[i][0] * ux + LGD_D3Q19_E[i][1] * uy + LGD_D3Q19_E[i][2] * uz;
        const double wi = (i < 7) ? w1 : w2;
        out[i] = keep * f[i] + wi * (d + eu + 1.5 * (eu * eu));
    }
}

/* The same collision for two cells at once (GCC vector extension: each
 * lane does the scalar function's operations in the same order, so the
 * results are the scalar ones bit for bit; the compiler maps the pairs to
 * SIMD registers, as the reference's updateLineX does with short_vec). */
typedef double lgd_v2d __attribute__((vector_size(16)));

static inline void lgd_d3q19_collide_v2(const lgd_v2d *f, double omega, lgd_v2d *out)
{
    lgd_v2d rho = {0.0, 0.0};
    int i;
    for (i = 0; i < 19; ++i) {
        rho += f[i];
    }
    const lgd_v2d ux =
        (f[LGD_Q_E] + f[LGD_Q_NE] + f[LGD_Q_SE] + f[LGD_Q_TE] + f[LGD_Q_BE]) -
        (f[LGD_Q_W] + f[LGD_Q_NW] + f[LGD_Q_SW] + f[LGD_Q_TW] + f[LGD_Q_BW]);
    const lgd_v2d uy =
        (f[LGD_Q_N] + f[LGD_Q_NW] + f[LGD_Q_NE] + f[LGD_Q_TN] + f[LGD_Q_BN]) -
        (f[LGD_Q_S] + f[LGD_Q_SW] + f[LGD_Q_SE] + f[LGD_Q_TS] + f[LGD_Q_BS]);
    const lgd_v2d uz =
        (f[LGD_Q_T] + f[LGD_Q_TW] + f[LGD_Q_TE] + f[LGD_Q_TN] + f[LGD_Q_TS]) -
        (f[LGD_Q_B] + f[LGD_Q_BW] + f[LGD_Q_BE] + f[LGD_Q_BN] + f[LGD_Q_BS]);
    const lgd_v2d usq = ux * ux + uy * uy + uz * uz;
    const lgd_v2d d = rho * (1.0 / 3.0) - 0.5 * usq;
    const double keep = 1.0 - omega;
    const double w1 = omega * (1.0 / 6.0);
    const double w2 = omega * (1.0 / 12.0);

    out[LGD_Q_C] = keep * f[LGD_Q_C] + omega * d;
    for (i = 1; i < 19; ++i) {
        const lgd_v2d eu = LGD_D3Q19_E[i][0] * ux + LGD_D3Q19_E[i][1] * uy + LGD_D3Q19_E[i][2] * uz;
        const double wi = (i < 7) ? w1 : w2;
        out[i] = keep * f[i] + wi * (d + eu + 1.5 * (eu * eu));
    }
}

#endif
