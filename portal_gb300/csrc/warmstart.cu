// Node features of the learned warm start (no reference counterpart).
//
// For every node, from the cloud and the device-resident radiation field of
// the last portal_radiation_field call (normally the pass over the starting
// populations):
//   0  log10 n_H2 [cm^-3]
//   1  log10 T_kin [K]
//   2  log10 |grad v| [s^-1]: Frobenius norm of the least-squares velocity
//      gradient over the node's Delaunay neighbours
//   3  cos^2 of the angle between the magnetic field and the local J^2_0
//      axis of line 1: the principal axis (largest |eigenvalue|) of the
//      traceless part of the field's second moment sum_rays w I n n, whose
//      five components are J^2_Q in any frame -- J^2_0 is extremal along it.
//      The reference forms J^2_0 in each node's field frame only
//      (inverse_rt.f90:128-129), so this direction has no counterpart there.
//   4  log10 J^0_0 / B_nu(T_kin) of line 1
//   5  log10 J^0_0 / B_nu(T_kin) of line 2 (line 1 again for one-line molecules)
//   6  100 J^2_0 / J^0_0 of line 1
//   7  100 J^2_0 / J^0_0 of line 2
#include <cmath>
#include <vector>

#include "common.cuh"

using namespace portal;

namespace {

__device__ double planck(double T, double nu) {
    if (T <= 0.0) return 0.0;
    return 1.4744995e-50 * nu * nu * nu / (exp(4.79924e-11 / T * nu) - 1.0);
}

__global__ void k_features(int N, int L, double tx, double nu0, double nu1, const double *__restrict__ pos,
                           const double *__restrict__ vel, const double *__restrict__ bvec,
                           const double *__restrict__ h2, const double *__restrict__ tk,
                           const int *__restrict__ off, const int *__restrict__ idx, const double *__restrict__ J0,
                           const double *__restrict__ J2, const float *__restrict__ km, float *__restrict__ F) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    // least-squares gradient G (3x3): G = R M^-1, M = sum dx dx^T, R = sum dv dx^T
    double Mx[9] = {0}, R[9] = {0};
    const double *xc = pos + 3 * (size_t)n, *vc = vel + 3 * (size_t)n;
    for (int q = off[n]; q < off[n + 1]; q++) {
        const int m = idx[q];
        double dx[3], dv[3];
        for (int k = 0; k < 3; k++) {
            dx[k] = (pos[3 * (size_t)m + k] - xc[k]) * tx;
            dv[k] = vel[3 * (size_t)m + k] - vc[k];
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                Mx[3 * i + j] += dx[i] * dx[j];
                R[3 * i + j] += dv[i] * dx[j];
            }
    }
    // inverse of the symmetric 3x3 M (cofactors)
    const double a = Mx[0], b = Mx[1], c = Mx[2], d = Mx[4], e = Mx[5], f = Mx[8];
    const double c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
    const double det = a * c00 + b * c01 + c * c02;
    double Mi[9] = {0};
    if (fabs(det) > 0.0) {
        Mi[0] = c00 / det; Mi[1] = c01 / det; Mi[2] = c02 / det;
        Mi[4] = (a * f - c * c) / det; Mi[5] = (b * c - a * e) / det;
        Mi[8] = (a * d - b * b) / det;
        Mi[3] = Mi[1]; Mi[6] = Mi[2]; Mi[7] = Mi[5];
    }
    // |G|^2 of the velocity gradient G = R Mi (Frobenius)
    double gn = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += R[3 * i + k] * Mi[3 * k + j];
            gn += s * s;
        }
    // the local J^2_0 axis: principal axis of the traceless second moment,
    // by power iteration on its square
    const double kxx = km[n], kyy = km[(size_t)N + n], kzz = km[2 * (size_t)N + n];
    const double kxy = km[3 * (size_t)N + n], kxz = km[4 * (size_t)N + n], kyz = km[5 * (size_t)N + n];
    const double tr3 = (kxx + kyy + kzz) / 3.0;
    const double S[9] = {kxx - tr3, kxy, kxz, kxy, kyy - tr3, kyz, kxz, kyz, kzz - tr3};
    double v[3] = {0.57735, 0.57735, 0.57735};
    for (int it = 0; it < 20; it++) {
        double w[3], u[3];
        for (int i = 0; i < 3; i++) w[i] = S[3 * i] * v[0] + S[3 * i + 1] * v[1] + S[3 * i + 2] * v[2];
        for (int i = 0; i < 3; i++) u[i] = S[3 * i] * w[0] + S[3 * i + 1] * w[1] + S[3 * i + 2] * w[2];
        const double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (!(un > 0.0)) break;
        for (int i = 0; i < 3; i++) v[i] = u[i] / un;
    }
    const double *bb = bvec + 3 * (size_t)n;
    const double cb = bb[0] * v[0] + bb[1] * v[1] + bb[2] * v[2];
    const double T = tk[n];
    const int l1 = (L > 1) ? 1 : 0;
    const double j00 = J0[(size_t)n * L], j01 = J0[(size_t)n * L + l1];
    const double b0 = planck(T, nu0), b1 = planck(T, nu1);
    float *o = F + 8 * (size_t)n;
    o[0] = (float)log10(fmax(h2[n] * 1e-6, 1e-30));
    o[1] = (float)log10(fmax(T, 1e-30));
    o[2] = (float)log10(sqrt(gn) + 1e-30);
    o[3] = (float)(cb * cb);
    o[4] = (float)log10(fmax(j00, 1e-300) / fmax(b0, 1e-300));
    o[5] = (float)log10(fmax(j01, 1e-300) / fmax(b1, 1e-300));
    o[6] = (float)(j00 != 0.0 ? 100.0 * J2[(size_t)n * L] / j00 : 0.0);
    o[7] = (float)(j01 != 0.0 ? 100.0 * J2[(size_t)n * L + l1] / j01 : 0.0);
}

}  // namespace

extern "C" int portal_warmstart_features(portal_ctx *c, float *features) {
    if (!c || !features) return PORTAL_ERR_ARG;
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    if (!c->j_valid) return set_err(c, PORTAL_ERR_STATE, "no device-resident radiation field");
    cudaSetDevice(c->device);
    const int N = c->N, L = c->r_num;
    DevBuf<float> F;
    if (F.reserve((size_t)N * 8)) return set_err(c, PORTAL_ERR_NOMEM, "features");
    if (!c->kmom.p) return set_err(c, PORTAL_ERR_STATE, "no radiation field computed");
    const double nu1 = c->nu[L > 1 ? 1 : 0];
    k_features<<<(N + 127) / 128, 128, 0, c->stream>>>(N, L, c->tx, c->nu[0], nu1, c->pos64.p, c->vel64.p,
                                                       c->bvec64.p, c->h2.p, c->tkin.p, c->nb_off.p, c->nb_idx.p,
                                                       c->J0.p, c->J2.p, c->kmom.p, F.p);
    PCHECK(c, cudaGetLastError());
    PCHECK(c, cudaMemcpyAsync(features, F.p, (size_t)N * 8 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    return PORTAL_OK;
}
