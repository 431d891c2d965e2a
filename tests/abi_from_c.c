/* Calls libgbns.so from plain C through include/gbns.h (no C++, no torch): the version, the
 * struct sizes, and an argument error with its message.  Built and run by tests/test_abi.py;
 * needs no GPU (no entry point below reaches a CUDA call). */
#include <stdio.h>
#include <string.h>
#include "gbns.h"

int main(void) {
    long long sz[6];
    if (gbns_version() != GBNS_VERSION) return 1;
    if (gbns_abi_sizes(sz, 6) != 0) return 2;
    if (sz[0] != (long long)sizeof(gbns_term_cond) || sz[1] != (long long)sizeof(gbns_evcalc) ||
        sz[2] != (long long)sizeof(gbns_run_desc) || sz[3] != (long long)sizeof(gbns_run_state) ||
        sz[4] != (long long)sizeof(gbns_batch) || sz[5] != (long long)sizeof(gbns_results_bufs))
        return 3;
    if (gbns_batch_iterate(NULL, 1, NULL) != -1) return 4;
    if (strstr(gbns_last_error(), "NULL") == NULL) return 5;
    if (gbns_threefry_split(NULL, NULL, 4, NULL) != -1) return 6;
    printf("ok %d %lld %lld\n", gbns_version(), sz[2], sz[4]);
    return 0;
}
