/* A C client of the library's C ABI (include/p9idg.h) with nothing in between: it reads a small
 * observation from raw little-endian files, partitions it (Partitioner.CreatePartition), grids
 * it with w-stacking (IDG.GridW), degrids a model grid (IDG.DeGridW, which shifts the grid in
 * place) and writes every result back as raw files, the way a P/Invoke shim would drive the
 * library.  tests/test_c_client.py builds it with gcc and checks the files against the FP64
 * oracle.
 *
 * usage: c_abi_client DIR nbl nt nch grid_size subgrid_size kernel_size max_timesteps
 *                     wlayer_count wstep scale vis_count mode
 * inputs:  DIR/uvw.bin double[nbl][nt][3], DIR/freq.bin double[nch],
 *          DIR/vis.bin complex128[nbl][nt][nch], DIR/grid.bin complex128[N][N]
 * outputs: DIR/subgrids.bin p9idg_subgrid[n], DIR/layers.bin complex128[W][N][N],
 *          DIR/vis_out.bin complex128[nbl][nt][nch], DIR/grid_shifted.bin complex128[N][N]
 * exit: 0 done; 3 no CUDA device (after subgrids.bin is written); 2 usage or file error;
 *       4 an ABI check failed; 10 + status for a failed call. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "p9idg.h"

static const char *g_dir;

static void *read_file(const char *name, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", g_dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    void *p = malloc(bytes ? bytes : 1);
    if (p && fread(p, 1, bytes, f) != bytes) {
        free(p);
        p = NULL;
    }
    fclose(f);
    return p;
}

static int write_file(const char *name, const void *p, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", g_dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) return 0;
    const int ok = fwrite(p, 1, bytes, f) == bytes;
    return fclose(f) == 0 && ok;
}

static int failed(const char *what, p9idg_status st) {
    fprintf(stderr, "%s: status %d: %s\n", what, (int)st, p9idg_last_error());
    return 10 + (int)st;
}

int main(int argc, char **argv) {
    if (argc != 14) {
        fprintf(stderr, "usage: %s DIR nbl nt nch N S kernel max_t W wstep scale vis_count mode\n", argv[0]);
        return 2;
    }
    g_dir = argv[1];
    const int32_t nbl = atoi(argv[2]), nt = atoi(argv[3]), nch = atoi(argv[4]);
    p9idg_params c;
    memset(&c, 0, sizeof c);
    c.grid_size = atoi(argv[5]);
    c.subgrid_size = atoi(argv[6]);
    c.kernel_size = atoi(argv[7]);
    c.max_timesteps = atoi(argv[8]);
    c.wlayer_count = atoi(argv[9]);
    c.wstep = strtod(argv[10], NULL);
    c.scale_arcsec = strtof(argv[11], NULL);
    c.vis_count = strtoll(argv[12], NULL, 10);
    const int32_t mode = atoi(argv[13]);
    const size_t nvis = (size_t)nbl * nt * nch, nn = (size_t)c.grid_size * c.grid_size;

    double *uvw = read_file("uvw.bin", sizeof(double) * 3 * nbl * nt);
    double *freq = read_file("freq.bin", sizeof(double) * nch);
    double *vis = read_file("vis.bin", sizeof(double) * 2 * nvis);
    double *grid = read_file("grid.bin", sizeof(double) * 2 * nn);
    if (!uvw || !freq || !vis || !grid) {
        fprintf(stderr, "missing input files in %s\n", g_dir);
        return 2;
    }

    /* the ABI's own checks: a null plan is an invalid argument, with a message */
    if (p9idg_grid_w(NULL, vis, uvw, vis) != P9IDG_INVALID_ARGUMENT || p9idg_last_error()[0] == '\0') {
        fprintf(stderr, "a null plan was not refused\n");
        return 4;
    }

    p9idg_plan *plan = NULL;
    p9idg_status st = p9idg_plan_create(&c, uvw, nbl, nt, freq, nch, &plan);
    if (st != P9IDG_OK) return failed("p9idg_plan_create", st);
    int64_t nsub = 0;
    if ((st = p9idg_plan_num_subgrids(plan, &nsub)) != P9IDG_OK) return failed("p9idg_plan_num_subgrids", st);
    p9idg_subgrid *subs = malloc(sizeof(p9idg_subgrid) * (size_t)(nsub > 0 ? nsub : 1));
    if ((st = p9idg_plan_get_subgrids(plan, subs, nsub)) != P9IDG_OK) return failed("p9idg_plan_get_subgrids", st);
    if (!write_file("subgrids.bin", subs, sizeof(p9idg_subgrid) * (size_t)nsub)) return 2;

    double *layers = calloc(2 * nn * (size_t)(c.wlayer_count > 0 ? c.wlayer_count : 1), sizeof(double));
    double *vis_out = calloc(2 * nvis, sizeof(double));
    st = p9idg_plan_set_mode(plan, mode);
    if (st == P9IDG_OK) st = p9idg_grid_w(plan, vis, uvw, layers);
    if (st == P9IDG_NO_DEVICE) {
        fprintf(stderr, "no CUDA device: %s\n", p9idg_last_error());
        p9idg_plan_destroy(plan);
        return 3;
    }
    if (st != P9IDG_OK) return failed("p9idg_grid_w", st);
    if (!write_file("layers.bin", layers, sizeof(double) * 2 * nn * (size_t)c.wlayer_count)) return 2;
    if ((st = p9idg_degrid_w(plan, grid, uvw, vis_out)) != P9IDG_OK) return failed("p9idg_degrid_w", st);
    if (!write_file("vis_out.bin", vis_out, sizeof(double) * 2 * nvis)) return 2;
    if (!write_file("grid_shifted.bin", grid, sizeof(double) * 2 * nn)) return 2;
    p9idg_plan_info info;
    if ((st = p9idg_plan_get_info(plan, &info)) != P9IDG_OK) return failed("p9idg_plan_get_info", st);
    printf("subgrids %lld gridded %lld of %lld mode %d\n", (long long)info.num_subgrids,
           (long long)info.gridded_visibilities, (long long)info.input_visibilities, (int)info.mode);
    p9idg_plan_destroy(plan);
    free(uvw);
    free(freq);
    free(vis);
    free(grid);
    free(subs);
    free(layers);
    free(vis_out);
    return 0;
}
