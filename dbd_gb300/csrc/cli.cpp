// cli.cpp -- bin/SSpMM, bin/compute, bin/d2h and bin/debug: the reference's
// executables (ZIP:dbd/Makefile:17-30) as callers of libdbd.
//
// Same argv (ZIP:dbd/src/main.cpp:152-187): A | A B | cpuGiB gpuGiB A |
// cpuGiB gpuGiB A B, budgets in GiB (default 28 / 22).  Same outputs: old
// Ptr.output / Idx.output / Val.output are removed first (main.cpp:62-64),
// the product is written to the working directory by bin/SSpMM and bin/debug,
// and the timing block of main.cpp:100-106 is printed.  The scope is fixed at
// build time: -DDBD_CLI_SCOPE=0 (compute), 1 (d2h), 2 (SSpMM, debug).
//
// The output files keep the reference's layout by default: float32
// Val.output (values computed in FP64, rounded on write) and int32
// Ptr.output, which becomes int64 only when nnz(C) >= 2^31, where the
// reference's own int32 ptrC wraps (distributeWorkload.cpp:207-212).
// DBD_OUT_FP64=1 writes this library's FP64 values and int64 row pointers.
// Further switches: DBD_ROWS_IN_BLOCK selects 4096 (for_small_datasets,
// default) or 512 (for_large_datasets) instead of two builds;
// DBD_IO_BUFFERED=1 writes through the page cache instead of O_DIRECT;
// DBD_IO_RESUME=1 keeps a progress manifest and continues an interrupted
// run; DBD_JSON=1 adds one JSON line.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/dbd.h"

#ifndef DBD_CLI_SCOPE
#define DBD_CLI_SCOPE 2
#endif

static void usage_and_exit() {
    puts("Invalid Arguments.");
    puts("Usage:\t<1> Executable File Name, Input File 1");
    puts("\t<2> Executable File Name, Input File 1, Input File 2");
    puts("\t<3> Executable File Name, CPU DRAM Size, GPU DRAM Size, Input File 1");
    puts("\t<4> Executable File Name, CPU DRAM Size, GPU DRAM Size, Input File 1, Input File 2\n");
    exit(-1);
}

static double env_num(const char *name, double dflt) {
    const char *v = getenv(name);
    return (v && *v) ? atof(v) : dflt;
}

int main(int argc, char **argv) {
    puts("\nLarge-Scaled Sparse Matrix - Sparse Matrix Multiplication. (L3SpMM)\n");
    remove("Ptr.output");
    remove("Idx.output");
    remove("Val.output");

    dbd_config cfg;
    dbd_config_default(&cfg);
    std::string fa, fb;
    if (argc == 2) {
        fa = fb = argv[1];
    } else if (argc == 3) {
        fa = argv[1];
        fb = argv[2];
    } else if (argc == 4) {
        cfg.host_gib = atoi(argv[1]);
        cfg.gpu_gib = atoi(argv[2]);
        fa = fb = argv[3];
    } else if (argc == 5) {
        cfg.host_gib = atoi(argv[1]);
        cfg.gpu_gib = atoi(argv[2]);
        fa = argv[3];
        fb = argv[4];
    } else {
        usage_and_exit();
    }
    cfg.rows_per_block = (int64_t)env_num("DBD_ROWS_IN_BLOCK", 4096);
    const bool fp64 = env_num("DBD_OUT_FP64", 0) != 0;
    cfg.out_val_fp32 = fp64 ? 0 : 1;
    cfg.out_ptr32 = fp64 ? 0 : 2;
    cfg.io_buffered = (int)env_num("DBD_IO_BUFFERED", 0);
    cfg.io_resume = (int)env_num("DBD_IO_RESUME", 0);
    cfg.io_rotate_gib = env_num("DBD_IO_ROTATE_GIB", 0);
    cfg.device = (int)env_num("DBD_DEVICE", 0);
    cfg.verbose = 1;

    dbd_ctx *ctx = nullptr;
    int rc = dbd_create(&cfg, &ctx);
    if (rc) {
        fprintf(stderr, "dbd_create: %s\n", dbd_error_string(rc));
        return 1;
    }
    dbd_stats st;
    memset(&st, 0, sizeof(st));
    rc = dbd_spgemm_files(ctx, fa.c_str(), fa == fb ? nullptr : fb.c_str(), (dbd_scope)DBD_CLI_SCOPE, ".", &st);
    if (rc) {
        fprintf(stderr, "%s: %s\n", dbd_error_string(rc), dbd_last_error(ctx));
        dbd_destroy(ctx);
        return 1;
    }
    printf("%f\n", st.t_kernel_exec);
    printf(" - Workload Distribution -\nCPUs\tBlocks:   %d (%.2f %%)\n\tElements: %ld (%.2f %%)\n", 0, 0.0, 0L, 0.0);
    printf("GPUs\tBlocks:   %lld (%.2f %%)\n\tElements: %lld (%.2f %%)\n\n", (long long)st.n_blocks, 100.0,
           (long long)st.products, 100.0);
    printf("------------ AVG TIME ------------\n");
    printf("Preprocessing\t\t%f s\n", st.t_preprocess);
    printf("Compute CPU\t\t%f s\n", 0.0);
    printf("Compute GPU\t\t%f s\n", st.t_compute_gpu);
    printf("Write File\t\t%f s\n", st.t_write_file);
    printf("Kernel Execution\t%f s\n", st.t_kernel_exec);
    printf("Total Execution\t\t%f s\n", st.t_total);
#ifdef DBD_CLI_DEBUG
    puts("\n - DEBUG -");
    printf("Top 10%% (Higher than %d): %lld\n", st.criteria, (long long)st.blocks_per_category[0]);
    printf("Lower than Two Warp Size (64): %lld\n", (long long)st.blocks_per_category[1]);
    printf("Computed Total %lld Elements\n", (long long)st.products);
    printf("Actual Total %lld Elements\n", (long long)st.nnz_c);
    printf("Reduced to %.2f %% After Merge\n", st.products ? 100.0 * st.nnz_c / st.products : 0.0);
    printf("Output chunks: %d; numeric rows per bin: empty %lld tiny %lld warp %lld ctaS %lld ctaL %lld dense %lld\n",
           st.n_chunks, (long long)st.rows_per_bin[0], (long long)st.rows_per_bin[1], (long long)st.rows_per_bin[2],
           (long long)st.rows_per_bin[3], (long long)st.rows_per_bin[4], (long long)st.rows_per_bin[5]);
#endif
    if (env_num("DBD_JSON", 0) != 0) {
        const double t = st.t_total > 0 ? st.t_total : 1e-30;
        printf("{\"scope\": %d, \"products\": %lld, \"nnz_c\": %lld, \"t_total_s\": %.9f, \"t_kernel_exec_s\": %.9f, "
               "\"t_preprocess_s\": %.9f, \"t_device_ms\": %.6f, \"t_fsync_s\": %.6f, \"gflops\": %.4f}\n",
               DBD_CLI_SCOPE, (long long)st.products, (long long)st.nnz_c, st.t_total, st.t_kernel_exec,
               st.t_preprocess, st.t_device_ms, st.t_fsync, 2.0 * (double)st.products / t / 1e9);
    }
    dbd_destroy(ctx);
    return 0;
}
