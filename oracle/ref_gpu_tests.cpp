// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// The reference's own GPU test, run against this repository's module: the
// reference's test translation unit (tests/test_kinetics.cpp, compiled from the
// reference sources by include path, nothing copied) with its `main` renamed,
// and a main here that performs the original main's set-up
// (test_kinetics.cpp:1051-1060) and then calls only its test_gpu
// (test_kinetics.cpp:1086-1243) -- the CPU-only tests of that file are the
// reference's business and take minutes.
//
// test_gpu loads `simstack_gpu.so` from this executable's directory with the
// reference's own loader (platform/linux_gpu.cpp:7-31); oracle/Makefile puts a
// symbolic link there to simstack_gb300/libsimstack_gpu.so. It checks, bit for
// bit against the reference's CPU lanes on the same host: FP64 and f32 lanes in
// both discharge modes, ten 20 ms steps with uploads every step, the
// warp-per-zone mode (gpu_kin_set_mode(1)), and the hybrid CPU+GPU driver
// (dbd.cpp:336-463) with the lanes split 0/8/24/40/64 of 64 zones between the
// module and the reference's own threaded CPU path. Exit code = failed checks.
// With --bench it also runs test_gpu's timing table (test_kinetics.cpp:1244-1298:
// 64-16,384 zones, per 1 ms master step, the module's FP64 / f32 thread / f32 warp
// paths against one CPU core), the harness behind the reference's published GPU
// figures.

#define main reference_test_kinetics_main
#include "tests/test_kinetics.cpp"
#undef main

int main(int argc, char **argv) {
    b32 bench = argc > 1 && strcmp(argv[1], "--bench") == 0;
    KinModel *model = (KinModel *)calloc(1, sizeof(KinModel));
    AirSpecies sp;
    air_mech_build(model, &sp);
    AirSourceModel src = air_source_defaults();
    test_mechanism(model);
    test_gpu(model, &sp, &src, bench);
    printf("%u checks, %u failed (simd=%d)\n", g_checks, g_failures, SIM_SIMD);
    free(model);
    return (int)g_failures;
}
