/* Prints the size and every member offset of the C ABI's structs (include/feynsimul.h) as
 * "struct member offset" lines, for the test that holds the Python ctypes mirrors to them. */
#include <stddef.h>
#include <stdio.h>

#include "feynsimul.h"

#define OFF(T, m) printf(#T " " #m " %zu\n", offsetof(T, m))

int main(void)
{
    printf("fs_config sizeof %zu\n", sizeof(fs_config));
    OFF(fs_config, dof); OFF(fs_config, n_slices); OFF(fs_config, bisection_level); OFF(fs_config, beta);
    OFF(fs_config, n_walkers); OFF(fs_config, walkers_per_group); OFF(fs_config, operator_runs);
    OFF(fs_config, metro_steps_per_operator_run); OFF(fs_config, enable_parallelize_path);
    OFF(fs_config, enable_ranlux); OFF(fs_config, luxury_factor); OFF(fs_config, ranlux_int_max);
    OFF(fs_config, enable_double); OFF(fs_config, enable_bins); OFF(fs_config, x_min); OFF(fs_config, x_max);
    OFF(fs_config, bin_resolution_per_dof); OFF(fs_config, hist_lo); OFF(fs_config, hist_hi);
    OFF(fs_config, hist_bins); OFF(fs_config, compat); OFF(fs_config, accum); OFF(fs_config, partials);
    OFF(fs_config, fast_math); OFF(fs_config, walkers_per_block); OFF(fs_config, min_blocks_per_sm);
    OFF(fs_config, learned); OFF(fs_config, global_path); OFF(fs_config, potential_cache); OFF(fs_config, moves);
    OFF(fs_config, alpha); OFF(fs_config, ps_alpha);
    printf("fs_info sizeof %zu\n", sizeof(fs_info));
    OFF(fs_info, n_threads); OFF(fs_info, threads_per_walker); OFF(fs_info, walkers_per_block);
    OFF(fs_info, block_threads); OFF(fs_info, grid_blocks); OFF(fs_info, smem_bytes); OFF(fs_info, registers);
    OFF(fs_info, device_bytes); OFF(fs_info, uniforms_per_move); OFF(fs_info, nodes_per_move);
    OFF(fs_info, potential_cache);
    printf("fs_batch_system sizeof %zu\n", sizeof(fs_batch_system));
    OFF(fs_batch_system, type); OFF(fs_batch_system, n_walkers); OFF(fs_batch_system, n_slices);
    OFF(fs_batch_system, bisection_level); OFF(fs_batch_system, beta); OFF(fs_batch_system, walkers_per_tile);
    return 0;
}
