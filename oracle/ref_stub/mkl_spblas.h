/* Empty stand-in for MKL's sparse BLAS header: the reference includes it in
 * src/util/hhp_cpu.c:10 but only commented-out code uses it. Test infrastructure. */
