/*
 * geokerr_c_api.h -- C ABI of the GB300 GEOKERR-equivalent Mino-time solver.
 *
 * Drop-in for the reference's geokerr_port C interfaces:
 *   geokerr_eval_lambda, geokerr_estimate_periods, geokerr_phi_omega
 *       Fortran ISO_C_BINDING entry points, geokerr_port/reference/
 *       geokerr_eval_lambda.f90:57-70, 205-210, 299-306 (C prototypes used
 *       by the reference at geokerr_port/validation/gkval_adapters.c:33-44);
 *   geokerr_stream_cuda, geokerr_complete_stream_cuda
 *       CUDA host wrappers, geokerr_port/cuda/geokerr_stream.cu:158-161 and
 *       geokerr_port/cuda/geokerr_complete.cu:446-449;
 *   compute_geokerr_complete_cuda
 *       geokerr_port/cuda/geokerr_complete.cu:356-363.
 * Same names, argument order and meaning, host pointers, synchronous; the
 * work runs on the current CUDA device.  Units M = E = 1, u = 1/r,
 * mu = cos(theta), Lz = L/E, Q2 = Q/E^2.
 *
 * The batched entry points (np_geokerr_*) take device pointers, run one
 * geodesic per GPU thread and return np_status codes (include/np_render.h).
 */
#ifndef GEOKERR_C_API_H
#define GEOKERR_C_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Samples one null geodesic at S affine parameters lam0 + k dlam
 * (geokerr_eval_lambda.f90:57-203): GEOKERR's NUP = S points uniform in u
 * (OFFSET 0.5, in to the radial turning point and back), linearly resampled
 * in affine lambda; u, mu at k = 0 are forced to the inputs; tpmi/tpri are
 * the 0-based grid indices of the first mu / u turning points or -1;
 * info = 0 ok, 1 if S <= 0, 2 if the geodesic could not be sampled. */
void geokerr_eval_lambda(double u0, double mu0, double uf, double a, double Lz, double Q2, double t0,
                         double lam0, double dlam, int S,
                         double* u, double* mu, double* t, double* phi, double* affine,
                         int* tpmi, int* tpri, int* info);

/* Radial and polar periods in affine lambda from turning-point spacing on a
 * 4096-point sampling (geokerr_eval_lambda.f90:205-297); -1 when not found. */
void geokerr_estimate_periods(double u0, double mu0, double a, double Lz, double Q2,
                              double* Tr, double* Ttheta, int* info);

/* d phi / d lambda (Mino) at (u0, mu0) (geokerr_eval_lambda.f90:299-306). */
double geokerr_phi_omega(double u0, double mu0, double a, double Lz, double Q2);

/* Exact Mino-time samples lambda_k = lam0 + k dlam (k < S) of the geodesic
 * leaving u0 towards uf (du/dlambda sign from uf - u0, dmu/dlambda sign -1
 * for mu0 > 0): u, mu, t, phi and lambda itself in h_affine.  Returns 0,
 * -1 bad argument, -2 allocation failure, -3 kernel failure
 * (geokerr_stream.cu:163-180). */
int geokerr_stream_cuda(double u0, double uf, double mu0, double a, double L, double Q2,
                        double lam0, double dlam, int S,
                        double* h_u, double* h_mu, double* h_t, double* h_phi, double* h_affine);

/* geokerr_eval_lambda on the GPU (the gkval harness's CUDA solver,
 * gkval_adapters.c:675-682); t0 = 0.  Return codes as geokerr_stream_cuda. */
int geokerr_complete_stream_cuda(double u0, double uf, double mu0, double a, double L, double Q2,
                                 double lam0, double dlam, int S,
                                 double* h_u, double* h_mu, double* h_t, double* h_phi, double* h_affine);

/* Per ray i < n: Mino time lambda from u0 to uf (through the radial turning
 * point when uf lies beyond it, GEOMU semantics), mu at uf, a case number
 * (1 turning point on the way in, 2 turning point on the way out, 3 no
 * turning point) and a validity flag. */
void compute_geokerr_complete_cuda(const double* h_u0, const double* h_uf, const double* h_mu0,
                                   const double* h_a, const double* h_l, const double* h_q2,
                                   const int* h_su, const int* h_sm,
                                   double* h_lambda_results, double* h_muf_results,
                                   int* h_ncase_results, char* h_valid_results, int n_cases);

/* Final state after Mino time lambda_max (geokerr_port/cuda/geokerr_cuda.cu:
 * 319-323 and geokerr_improved.cu:378-382, whose bodies there are
 * placeholders): ray i with spin a_vals[i] starts at r0_vals[i],
 * mu0_vals[i] with E_vals[i] > 0, L_vals[i], Q2_vals[i] (any normalisation),
 * outgoing in r and increasing in mu as those wrappers integrate; outputs
 * r, mu, phi and t (phi, t from 0) at Mino time lambda_max of that
 * normalisation, integrated exactly by the Mino-time solver (n_steps is
 * accepted and not needed).  A ray that reaches the horizon or r = infinity
 * first keeps its last state there; a forbidden start gives NaN.  Both
 * names run the same solver. */
void geokerr_cuda_batch(const double* a_vals, const double* r0_vals, const double* mu0_vals,
                        const double* E_vals, const double* L_vals, const double* Q2_vals,
                        double* r_final, double* mu_final, double* phi_final, double* t_final,
                        int n_geodesics, int n_steps, double lambda_max);
void geokerr_improved_batch(const double* a_vals, const double* r0_vals, const double* mu0_vals,
                            const double* E_vals, const double* L_vals, const double* Q2_vals,
                            double* r_final, double* mu_final, double* phi_final, double* t_final,
                            int n_geodesics, int n_steps, double lambda_max);

/* Mino time from u0 to uf (geokerr_port/cuda/mino_time_cuda.cu:270-280, a
 * placeholder there): the radial motion with sign su[i] reaching uf[i]
 * directly (tpr[i] = 0) or after its radial turning point (tpr[i] = 1).
 * lambda is fixed by the radial motion, so muf, tpm and ncase are accepted
 * and not needed; valid[i] = 0 when uf is not reached that way. */
void compute_mino_time_batch_cuda(const double* h_u0, const double* h_uf, const double* h_mu0,
                                  const double* h_muf, const double* h_a, const double* h_l,
                                  const double* h_q2, const int* h_tpm, const int* h_tpr,
                                  const int* h_su, const int* h_sm, const int* h_ncase,
                                  double* h_lambda_results, char* h_valid_results, int n_cases);

/* The Fortran single-case entry (geokerr_port/reference/geokerr_single.f:1-3,
 * called by geokerr_compare.cu:27-33), arguments by reference: Mino time
 * from u0 to uf and mu there, as compute_geokerr_complete_cuda for one ray
 * (muf is accepted and not needed). */
void geokerr_single_case_(double* u0, double* uf, double* mu0, double* muf, double* a, double* l, double* q2,
                          int* su, int* sm, double* lambda, double* muf_out, int* ncase, int* valid);

/* State at Mino time lam[i] of ray i (spin a[i]) leaving (u0[i], mu0[i])
 * with signs su[i], sm[i] of du/dlambda and dmu/dlambda: u, mu, t and phi
 * (t and phi from 0); valid[i] = 0 when the ray reached the horizon or
 * u = 0 first (the last state before it is returned) or started in a
 * forbidden region (NaN).  Host arrays; returns np_status. */
int np_geokerr_final_state_host(int n, const double* a, const double* u0, const double* mu0, const double* l,
                                const double* q2, const double* su, const double* sm, const double* lam,
                                double* u, double* mu, double* t, double* phi, char* valid);

/* Batched GEOKERR sampler (geokerr_original.f:357-605 with USEGEOR false,
 * PHIT true, NPTS = 0): ray i uses u0[i], uf[i], mu0[i], l[i], q2[i],
 * su[i], sm[i] and the common spin a, TPR flag, nup and offset; outputs are
 * [n][nup] device arrays (u, mu, delta t, delta phi, affine lambda, mu and
 * u turning counts) and npts[i] = points written (0 when the ray could not
 * be sampled).  Every point is evaluated in closed form by its own thread
 * (the semi-analytic GEOR / GEOMU / GEOPHITIME route,
 * geokerr_original.f:771-1187, 1648-2360); rays outside the closed forms
 * (q2 = 0, a = 0, a double radial root) are integrated by the order-24
 * Taylor solver.  n * nup < 2^31.  Device pointers; the per-ray workspace
 * comes from the stream-ordered allocator.  Returns np_status. */
int np_geokerr_points_device(int n, double a, const double* u0, const double* uf, const double* mu0,
                             const double* l, const double* q2, const double* su, const double* sm,
                             int tpr, int nup, double offset,
                             double* u, double* mu, double* dt, double* dphi, double* lam,
                             int32_t* tpm, int32_t* tprv, int32_t* npts, void* stream);

/* The same sampler with every ray on the Taylor solver (one thread per ray). */
int np_geokerr_points_taylor_device(int n, double a, const double* u0, const double* uf, const double* mu0,
                                    const double* l, const double* q2, const double* su, const double* sm,
                                    int tpr, int nup, double offset,
                                    double* u, double* mu, double* dt, double* dphi, double* lam,
                                    int32_t* tpm, int32_t* tprv, int32_t* npts, void* stream);

/* np_geokerr_points_device on the host (same arithmetic, same bits);
 * method[i] (optional) = 1 four real radial roots, 2 two real roots and a
 * complex pair around the motion, 3 two real roots below it and a complex
 * pair (q2 < 0), 4 two complex pairs (q2 < 0), 0 Taylor solver or no
 * points. */
int np_geokerr_points_host(int n, double a, const double* u0, const double* uf, const double* mu0,
                           const double* l, const double* q2, const double* su, const double* sm,
                           int tpr, int nup, double offset,
                           double* u, double* mu, double* dt, double* dphi, double* lam,
                           int32_t* tpm, int32_t* tprv, int32_t* npts, int32_t* method);

/* Batched geokerr_eval_lambda: ray i with u0[i], mu0[i], uf[i], Lz[i],
 * Q2[i], t0[i], lam0[i], dlam[i] and common a and S; outputs [n][S]
 * device arrays plus tpmi[n], tpri[n], info[n].  `work` is caller scratch
 * of at least np_geokerr_eval_lambda_work_bytes(n, S) bytes, or NULL to let
 * the library allocate it.  Returns np_status. */
int np_geokerr_eval_lambda_device(int n, double a, const double* u0, const double* mu0, const double* uf,
                                  const double* Lz, const double* Q2, const double* t0,
                                  const double* lam0, const double* dlam, int S,
                                  double* u, double* mu, double* t, double* phi, double* affine,
                                  int32_t* tpmi, int32_t* tpri, int32_t* info, void* work, void* stream);
size_t np_geokerr_eval_lambda_work_bytes(int n, int S);

/* Equatorial crossings (mu = 0; GEOR with muf = 0, geokerr_original.f:2672)
 * of rays leaving (u0[i], mu0[i]) with constants l[i], q2[i] and initial
 * signs su[i] (du/dlambda), sm[i] (dmu/dlambda): the first K crossings' u
 * and phi (phi measured from the start) in xu[n][K], xphi[n][K], their count
 * in nx[i] (-1 when the start is forbidden).  A ray ends at the horizon, at
 * u <= u_end or after K crossings.  Device pointers; returns np_status. */
int np_geokerr_equator_crossings_device(int n, double a, const double* u0, const double* mu0, const double* l,
                                        const double* q2, const double* su, const double* sm, double u_end, int K,
                                        double* xu, double* xphi, int32_t* nx, void* stream);

/* Carlson symmetric elliptic integrals, FP64 (Carlson 1995 duplication):
 * case i is types[2i..2i+1] = "RF" (x, y, z), "RC" (x, y), "RD" (x, y, z) or
 * "RJ" (x, y, z, p); R_C with y < 0 and R_J with p < 0 are Cauchy principal
 * values; invalid arguments or codes give NaN (the batch kernel of
 * geokerr_port/cuda/carlson_elliptic.cu:351-382).  d_p may be NULL when no
 * case is "RJ".  Device pointers, ordered on `stream`; the host entry runs the
 * same code on the CPU.  Both return np_status. */
int np_carlson_batch_device(int n, const char* d_types, const double* d_x, const double* d_y, const double* d_z,
                            const double* d_p, double* d_out, void* stream);
int np_carlson_batch_host(int n, const char* types, const double* x, const double* y, const double* z,
                          const double* p, double* out);
/* Semi-analytic Mino times with Carlson's R_F (E = 1, a the spin, l[i] =
 * L/E, q2[i] = Q/E^2): lam_u[i] = int du / sqrt(U(u)) from ua[i] to ub[i] and
 * lam_mu[i] = int dmu / sqrt(M(mu)) from mua[i] to mub[i], each on one
 * monotonic segment of the radial and polar motion (no turning point strictly
 * inside; endpoints may be turning points).  The radial form covers four
 * (three) real roots of U and one complex root pair, the polar form q2 > 0
 * (NaN otherwise).  Device
 * pointers on `stream`, or host pointers; np_status. */
int np_geokerr_mino_times_device(int n, double a, const double* d_ua, const double* d_ub, const double* d_mua,
                                 const double* d_mub, const double* d_l, const double* d_q2, double* d_lam_u,
                                 double* d_lam_mu, void* stream);
int np_geokerr_mino_times_host(int n, double a, const double* ua, const double* ub, const double* mua,
                               const double* mub, const double* l, const double* q2, double* lam_u, double* lam_mu);
/* Polar motion in closed form (q2[i] > 0): mu at Mino time lam[i] of the
 * geodesic with mu(0) = mu0[i] and sign sm[i] of dmu/dlambda at 0, through
 * any number of turning points: mu = mu_+ cn(omega lambda - sm F, k) with
 * Jacobi cn (AGM / descending Landen) and F from Carlson's R_F (the role of
 * GEOMU's Jacobi inversion, geokerr_original.f:1147-1178).  NaN for q2 <= 0. */
int np_geokerr_mu_of_lambda_device(int n, double a, const double* d_l, const double* d_q2, const double* d_mu0,
                                   const double* d_sm, const double* d_lam, double* d_mu, void* stream);
int np_geokerr_mu_of_lambda_host(int n, double a, const double* l, const double* q2, const double* mu0,
                                 const double* sm, const double* lam, double* mu);
/* Equatorial crossings in closed form (GEOR with mu_f = 0,
 * geokerr_original.f:2672-3136, semi-analytic): the polar motion gives each
 * crossing's Mino time, the radial Mino-time integral (Carlson R_F) is
 * inverted there.  Same rays, signs and stopping rules as
 * np_geokerr_equator_crossings_device; xu[n][K] only (no phi); nx[i] = -1
 * for q2[i] <= 0. */
int np_geokerr_equator_crossings_cf_device(int n, double a, const double* d_u0, const double* d_mu0, const double* d_l,
                                           const double* d_q2, const double* d_su, const double* d_sm, double u_end,
                                           int K, double* d_xu, int32_t* d_nx, void* stream);
int np_geokerr_equator_crossings_cf_host(int n, double a, const double* u0, const double* mu0, const double* l,
                                         const double* q2, const double* su, const double* sm, double u_end, int K,
                                         double* xu, int32_t* nx);
/* Equatorial crossings in closed form by Jacobi amplitude: the polar motion
 * mu = mu+ cn(omega lambda + w0 | k) gives the Mino time of each crossing,
 * the radial motion's Legendre variable S = sn^2(F | m) its u, one amplitude
 * per crossing (the crossings of GEOR with muf = 0, geokerr_original.f:
 * 2672-3136, without integration).  Per ray: the first K (1..16) crossings
 * with u in [u_lo, u_hi] along the ray to its end (the horizon, or u_far
 * after its radial turning point): u in xu[n][K], the azimuth change from
 * the start in xphi[n][K] (NULL to skip; NaN for a polar orbit through the
 * pole with l != 0), the count in nx[i] and in status[i] (NULL to skip) 0
 * (leaves through u_far), 1 (falls into the horizon) or -1 (outside the
 * closed forms: a = 0, q2 = 0, a start inside the photon region or inside
 * u_far, or a ray within ~1e-9 relative of the critical curve whose pair
 * of radial roots is not resolved).  q2 < 0 rays have no crossing.
 * np_status. */
int np_geokerr_disk_crossings_device(int n, double a, const double* d_u0, const double* d_mu0, const double* d_l,
                                     const double* d_q2, const double* d_su, const double* d_sm, double u_far,
                                     double u_lo, double u_hi, int K, double* d_xu, double* d_xphi, int32_t* d_nx,
                                     int32_t* d_status, void* stream);
int np_geokerr_disk_crossings_host(int n, double a, const double* u0, const double* mu0, const double* l,
                                   const double* q2, const double* su, const double* sm, double u_far, double u_lo,
                                   double u_hi, int K, double* xu, double* xphi, int32_t* nx, int32_t* status);
/* GEOKERR's standard camera grid (geokerr_original.f:183-220): n_alpha x
 * n_beta cell-centred image positions alpha = a1 + (a2 - a1)(i + 1/2) /
 * n_alpha, beta = b1 + (b2 - b1)(j + 1/2) / n_beta (ray index i n_beta + j),
 * and the constants of each ray: l = -alpha sqrt(1 - mu0^2), q2 = beta^2 -
 * (a^2 - alpha^2) mu0^2, snapped to 0 when |q2| < input_limit^2 or |l| <
 * input_limit (a snaps when |a| < input_limit); su = 1; sm = +1 when beta > 0
 * and mu0 < 1, else -1.  Output arrays of n_alpha n_beta doubles; the device
 * entry fills device arrays on `stream`, the host entry host arrays.
 * np_status (invalid sizes: NP_ERR_INVALID). */
int np_geokerr_camera_grid_device(double a, double mu0, int n_alpha, int n_beta, double a1, double a2, double b1,
                                  double b2, double input_limit, double* d_alpha, double* d_beta, double* d_l,
                                  double* d_q2, double* d_su, double* d_sm, void* stream);
int np_geokerr_camera_grid_host(double a, double mu0, int n_alpha, int n_beta, double a1, double a2, double b1,
                                double b2, double input_limit, double* alpha, double* beta, double* l, double* q2,
                                double* su, double* sm);
/* Jacobi elliptic functions sn, cn, dn(u[i] | m[i]), 0 <= m <= 1 (the role of
 * SNCNDN, geokerr_original.f:3277-3347), on the host. */
int np_jacobi_host(int n, const double* u, const double* m, double* sn, double* cn, double* dn);
/* The reference's host entry points (carlson_elliptic.cu:387, 398): a
 * device-vs-host check printed per function, and R_F(1, 2, 0) printed. */
void validate_carlson_cuda(void);
void test_carlson_cuda(void);

#ifdef __cplusplus
}
#endif

#endif /* GEOKERR_C_API_H */
