/* A C host of libfsi_gpu (tests/test_abi_symbols.py compiles it with
 * -std=c99 -pedantic -Werror and runs it without a GPU).
 *
 * It uses the header as a C program would: the descriptor filled field by
 * field, the opaque handles, the status codes and fsi_last_error. Every call
 * made here is refused by the library's argument checks before any CUDA
 * call, so the program runs on a host without a GPU; its output lists each
 * call's status and message for the test to compare. */
#include <stdio.h>
#include <string.h>

#include "fsi_gpu.h"

static void report(const char *what, int rc) {
    char msg[256];
    int n = fsi_last_error(msg, (int)sizeof msg);
    printf("%s %d %d %s\n", what, rc, n, msg);
}

int main(void) {
    fsi_block_desc d;
    fsi_block_t h = NULL;
    fsi_pair_t p = NULL;
    int k;

    memset(&d, 0, sizeof d);
    d.xDim = 16;
    d.yDim = 8;
    d.zDim = 8;
    d.dh = 1.0;
    for (k = 0; k < 6; k++) d.bndConds[k] = 101;
    d.iCollidModel = 12; /* RBGK: refused */
    d.nu = 0.01;
    d.precision = FSI_PREC_F64;
    d.denIn = 1.0;
    report("create_rbgk", fsi_block_create(&h, &d));
    d.iCollidModel = 13; /* ELBM: refused */
    report("create_elbm", fsi_block_create(&h, &d));
    d.iCollidModel = 1;
    d.xDim = 2; /* too small */
    report("create_small", fsi_block_create(&h, &d));
    report("create_null", fsi_block_create(NULL, &d));
    report("pair_null", fsi_pair_create(&p, NULL, NULL, 1));
    report("continue_null", fsi_continue_read("x", NULL, 1, NULL, NULL));
    report("destroy_null", fsi_block_destroy(NULL));
    return h == NULL && p == NULL ? 0 : 1;
}
