/*
 * include/nqs/nqs_gradient.h -- local-energy estimators.
 *
 * Drop-in for upstream include/nqs/nqs_gradient.h:39-101.  E_loc(s) =
 * sum_s' H_ss' psi(s')/psi(s); the connected configurations are enumerated
 * bit-exactly from bond tables and their amplitude ratios come from
 * incremental theta updates on the GPU.  Lattice conventions are upstream's:
 * site x*size_y + y; kagome passes unit cells and uses 3*size_x*size_y sites.
 * Square/chain lattices are open unless nqs_gpu_options_t.square_pbc is set.
 */
#ifndef NQS_GRADIENT_H
#define NQS_GRADIENT_H

#include "nqs_config.h"
#include "nqs_sampler.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces upstream nqs_local_energy (include/nqs/nqs_gradient.h:39).
 * Returns NaN (and sets nqs_gpu_last_error()) when the callback or the
 * Hamiltonian is not supported on the GPU; 0.0 on NULL arguments as upstream. */
double nqs_local_energy(const nqs_config_t *cfg,
                        int size_x, int size_y,
                        const int *spins,
                        nqs_log_amp_fn_t log_amp,
                        void *log_amp_user);

/* Replaces upstream nqs_local_energy_batch (include/nqs/nqs_gradient.h:46). */
void nqs_local_energy_batch(const nqs_config_t *cfg,
                            int size_x, int size_y,
                            const int *spins_batch, int batch_size,
                            nqs_log_amp_fn_t log_amp,
                            void *log_amp_user,
                            double *out_energies);

/* Replaces upstream nqs_local_energy_complex (include/nqs/nqs_gradient.h:59). */
void nqs_local_energy_complex(const nqs_config_t *cfg,
                               int size_x, int size_y,
                               const int *spins,
                               nqs_log_amp_fn_t log_amp,
                               void *log_amp_user,
                               double *out_re, double *out_im);

/* Replaces upstream nqs_local_energy_batch_complex (include/nqs/nqs_gradient.h:66). */
void nqs_local_energy_batch_complex(const nqs_config_t *cfg,
                                     int size_x, int size_y,
                                     const int *spins_batch, int batch_size,
                                     nqs_log_amp_fn_t log_amp,
                                     void *log_amp_user,
                                     double *out_re, double *out_im);

/* Running mean / variance accumulator, upstream include/nqs/nqs_gradient.h:73-101
 * (host-side helper, kept inline as upstream). */
typedef struct {
    double sum;
    double sum_sq;
    long   count;
} nqs_energy_accumulator_t;

static inline void nqs_energy_accumulator_init(nqs_energy_accumulator_t *a) {
    a->sum = 0.0;
    a->sum_sq = 0.0;
    a->count = 0;
}

static inline void nqs_energy_accumulator_add(nqs_energy_accumulator_t *a,
                                               double sample) {
    a->sum    += sample;
    a->sum_sq += sample * sample;
    a->count  += 1;
}

static inline double nqs_energy_accumulator_mean(const nqs_energy_accumulator_t *a) {
    return a->count > 0 ? a->sum / (double)a->count : 0.0;
}

static inline double nqs_energy_accumulator_variance(const nqs_energy_accumulator_t *a) {
    if (a->count < 2) return 0.0;
    double m = nqs_energy_accumulator_mean(a);
    return (a->sum_sq / (double)a->count) - m * m;
}

#ifdef __cplusplus
}
#endif

#endif /* NQS_GRADIENT_H */
