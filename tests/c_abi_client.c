/* A C caller of libnunatak_gb300 (no Python, no C++): reads the three descriptors as the bytes of their C
 * structs and the input fields as raw doubles from a directory, creates a context and a problem, sets the
 * fields, computes geometry and driving stress, runs picard_solve! and writes U and V back.  Used by
 * tests/test_c_abi.py: compiled on every machine (the header is plain C), run where a GPU is present. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nunatak_gb300.h"

static void* slurp(const char* dir, const char* name, size_t* bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    void* p = malloc(n > 0 ? (size_t)n : 1);
    if (p && fread(p, 1, (size_t)n, f) != (size_t)n) {
        free(p);
        p = NULL;
    }
    fclose(f);
    if (bytes) *bytes = (size_t)n;
    return p;
}

static int spit(const char* dir, const char* name, const void* p, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE* f = fopen(path, "wb");
    if (!f) return 1;
    size_t w = fwrite(p, 1, bytes, f);
    fclose(f);
    return w != bytes;
}

static int read_struct(const char* dir, const char* name, void* out, size_t size) {
    size_t n = 0;
    void* p = slurp(dir, name, &n);
    if (!p || n != size) {
        fprintf(stderr, "%s: expected %zu bytes, got %zu\n", name, size, n);
        free(p);
        return 1;
    }
    memcpy(out, p, size);
    free(p);
    return 0;
}

int main(int argc, char** argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s DIR\n", argv[0]);
        return 2;
    }
    const char* dir = argv[1];
    nk_grid_desc g;
    nk_physics_desc ph;
    nk_solver_desc sd;
    if (read_struct(dir, "grid.bin", &g, sizeof g) || read_struct(dir, "physics.bin", &ph, sizeof ph) ||
        read_struct(dir, "solver.bin", &sd, sizeof sd))
        return 2;
    g.x_faces = NULL;   /* regular axes and the default sigma faces: no pointers cross processes */
    g.y_faces = NULL;
    g.sigma_faces = NULL;

    nk_context* ctx = NULL;
    if (nk_context_create(0, &ctx) != NK_OK) {
        fprintf(stderr, "nk_context_create failed\n");
        return 3;
    }
    nk_problem* P = NULL;
    if (nk_problem_create(ctx, &g, &ph, &sd, &P) != NK_OK) {
        fprintf(stderr, "nk_problem_create: %s\n", nk_last_error(ctx));
        return 3;
    }
    const int32_t ids[3] = {NK_FIELD_H, NK_FIELD_BED, NK_FIELD_RATE_FACTOR};
    const char* names[3] = {"H.bin", "bed.bin", "A.bin"};
    for (int k = 0; k < 3; ++k) {
        size_t n = 0;
        double* a = (double*)slurp(dir, names[k], &n);
        if (!a || (int64_t)(n / sizeof(double)) != nk_problem_field_size(P, ids[k]) ||
            nk_problem_set_field(P, ids[k], a, (int64_t)(n / sizeof(double))) != NK_OK) {
            fprintf(stderr, "set %s: %s\n", names[k], nk_last_error(ctx));
            return 4;
        }
        free(a);
    }
    if (nk_compute_geometry(P) != NK_OK) {
        fprintf(stderr, "nk_compute_geometry: %s\n", nk_last_error(ctx));
        return 4;
    }
    nk_solve_stats st;
    nk_status s = nk_picard_solve(P, &st);
    printf("status %d picard_iterations %d linear_iterations_total %d\n", (int)s, (int)st.picard_iterations,
           (int)st.linear_iterations_total);
    int64_t nu = nk_problem_field_size(P, NK_FIELD_U), nv = nk_problem_field_size(P, NK_FIELD_V);
    double* u = (double*)malloc((size_t)nu * sizeof(double));
    double* v = (double*)malloc((size_t)nv * sizeof(double));
    if (nk_problem_get_field(P, NK_FIELD_U, u, nu) != NK_OK || nk_problem_get_field(P, NK_FIELD_V, v, nv) != NK_OK ||
        spit(dir, "u.bin", u, (size_t)nu * sizeof(double)) || spit(dir, "v.bin", v, (size_t)nv * sizeof(double))) {
        fprintf(stderr, "get u, v: %s\n", nk_last_error(ctx));
        return 5;
    }
    free(u);
    free(v);
    nk_problem_destroy(P);
    nk_context_destroy(ctx);
    return s == NK_OK ? 0 : 6;
}
