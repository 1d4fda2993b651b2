/* A plain C99 client of libcpm_gpu.so: host-only entry points (builder,
 * validation errors, theta length, derived seeds), as a C or Rust FFI caller
 * would use them. Compiled and run by tests/test_host_cpu.py. */
#include <stdio.h>
#include <string.h>
#include "cpm_gpu.h"

int main(void) {
    const uint64_t grid[2] = {30, 30};
    cpm_builder* b = NULL;
    if (cpm_builder_new(grid, 2, "periodic", 1, "von_neumann", NULL, "von_neumann", NULL, NULL, NULL, NULL, 0, &b)) {
        printf("new failed: %s\n", cpm_last_error());
        return 1;
    }
    if (cpm_builder_register_cell_type(b, "a", 50, 75, 10.0, 2.0, 0.0, 0)) return 2;
    if (cpm_builder_add_cells(b, "a", 5)) return 3;
    const double adh[4] = {0, 5, 5, 2};
    const size_t lens[2] = {2, 2};
    if (cpm_builder_set_adhesion(b, adh, lens, 2)) return 4;
    size_t n = 0;
    if (cpm_builder_theta_len(b, &n) || n != 7) return 5;
    int rc = cpm_builder_register_cell_type(b, "a", 50, 75, 10.0, 2.0, 0.0, 0);
    printf("dup rc=%d msg=%s\n", rc, cpm_last_error());
    printf("seed=%llu version=%s\n", (unsigned long long)cpm_derive_seed_u64(42, 0), cpm_version());
    cpm_builder_free(b);
    return rc == CPM_E_CONFIG ? 0 : 6;
}
