// w3o_umat.h -- TEST INFRASTRUCTURE ONLY (the oracle): the UMAT path of
// one material point (w3o_umat.cpp).
#pragma once

namespace w3o {

constexpr int UMAT_NSTATV = 20;   // umat_set_features info_vector(1) of the example UMAT
constexpr int UMAT_NPROPS = 50;

void umat_example(double* stress, double* statev, double* ddsdde, double& sse, double& spd, double* dstran,
                  const double* props, const double* drot, double dtemp);
bool umat_drive(const double* props, int step, int iter, bool extrapolated_du, const double* urcs_n,
                const double* eps_n, const double* uddt, const double* hist, int nstatv, double* urcs_n1,
                double* hist1, double* cep21);

}  // namespace w3o
