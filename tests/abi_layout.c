/* Prints sizeof and offsetof of every field of the structs in
 * include/baorec_gb300.h, one "struct field offset" line each, so that
 * tests/test_abi.py can compare the C layout with the ctypes mirror.
 * Compiled and run on the host by the test (no GPU). */
#include <stddef.h>
#include <stdio.h>

#include "baorec_gb300.h"

#define F(S, f) printf(#S " " #f " %zu\n", offsetof(S, f))
#define SZ(S) printf(#S " sizeof %zu\n", sizeof(S))

int main(void) {
  SZ(baorec_config);
  F(baorec_config, method); F(baorec_config, n); F(baorec_config, box_size); F(baorec_config, box_min);
  F(baorec_config, los_mode); F(baorec_config, los); F(baorec_config, bias); F(baorec_config, f);
  F(baorec_config, smoothing_radius); F(baorec_config, beta); F(baorec_config, n_iter);
  F(baorec_config, jacobi_damping_factor); F(baorec_config, jacobi_niterations);
  F(baorec_config, vcycle_niterations); F(baorec_config, ran_min); F(baorec_config, mas);
  F(baorec_config, mg_mode); F(baorec_config, nu1); F(baorec_config, nu2); F(baorec_config, rtol);
  F(baorec_config, max_cycles); F(baorec_config, mg_start); F(baorec_config, start_rate);
  SZ(baorec_solve_stats);
  F(baorec_solve_stats, cycles); F(baorec_solve_stats, spectral_steps); F(baorec_solve_stats, rel_residual);
  F(baorec_solve_stats, alpha); F(baorec_solve_stats, rel_residual_initial);
  SZ(baorec_batch_item);
  F(baorec_batch_item, x); F(baorec_batch_item, y); F(baorec_batch_item, z); F(baorec_batch_item, w);
  F(baorec_batch_item, n); F(baorec_batch_item, mesh); F(baorec_batch_item, box_size); F(baorec_batch_item, mas);
  F(baorec_batch_item, smoothing_radius); F(baorec_batch_item, field); F(baorec_batch_item, out_x);
  F(baorec_batch_item, out_y); F(baorec_batch_item, out_z);
  SZ(baorec_guess_train_config);
  F(baorec_guess_train_config, steps); F(baorec_guess_train_config, batch); F(baorec_guess_train_config, lr);
  F(baorec_guess_train_config, seed); F(baorec_guess_train_config, sigma_g); F(baorec_guess_train_config, pk_slope);
  F(baorec_guess_train_config, region_min); F(baorec_guess_train_config, region_size);
  F(baorec_guess_train_config, r_min); F(baorec_guess_train_config, r_max); F(baorec_guess_train_config, ra_min);
  F(baorec_guess_train_config, ra_max); F(baorec_guess_train_config, dec_min); F(baorec_guess_train_config, dec_max);
  F(baorec_guess_train_config, rtol); F(baorec_guess_train_config, loss);
  SZ(baorec_power_config);
  F(baorec_power_config, geometry); F(baorec_power_config, mas); F(baorec_power_config, interlace);
  F(baorec_power_config, nbins); F(baorec_power_config, kmin); F(baorec_power_config, dk);
  F(baorec_power_config, los); F(baorec_power_config, reserved);
  return 0;
}
