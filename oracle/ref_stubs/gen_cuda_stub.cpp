// Link-time stand-in for the reference's GPU entry point so that its CPU path
// (genDist -c) builds with g++ alone. Every invocation passes -c.
#include "genMain.h"
void computeGenDist_CUDA(FILE*, string, string, READ*&, int, int, float, int) {
    fprintf(stderr, "oracle/_ref genDist: GPU path not built; run with -c\n");
    exit(2);
}
