/*
 * The reference's makefile lists xc/vdW/vdWDF/vdWDFreadKernel.o, but that source file is not
 * in the reference tree. vdW-DF functionals are outside the oracle's use, so the one symbol
 * the rest of the program references is defined here and fails loudly if ever reached.
 */
#include <stdio.h>
#include <stdlib.h>

void vdWDF_read_kernel(void *pSPARC)
{
    (void)pSPARC;
    fprintf(stderr, "oracle: vdW-DF kernel reading is not part of this build\n");
    exit(EXIT_FAILURE);
}
