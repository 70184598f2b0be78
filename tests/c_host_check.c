/* Plain C host of libpq3d.so through include/pq3d.h only (no CUDA headers, no
 * Python): assembles the dense operator of a small planar mesh into host
 * buffers, evaluates the reference ABI TDstressFS_C at a few points, checks an
 * error return, and writes the results for the test to compare with the CPU
 * oracle.  Usage: c_host_check OUT.bin */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pq3d.h"

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    /* 4 x 3 squares of 1 km on the plane y = 0, two triangles each */
    const int nx = 4, nz = 3;
    const int64_t n_nodes = (nx + 1) * (nz + 1), N = 2 * nx * nz;
    double *nodes = (double *)malloc(sizeof(double) * 3 * n_nodes);
    int64_t *tris = (int64_t *)malloc(sizeof(int64_t) * 3 * N);
    for (int k = 0; k <= nz; ++k)
        for (int i = 0; i <= nx; ++i) {
            double *p = nodes + 3 * (k * (nx + 1) + i);
            p[0] = 1000.0 * i; p[1] = 0.0; p[2] = -1000.0 * (k + 1);
        }
    int64_t t = 0;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
            const int64_t a = k * (nx + 1) + i + 1, b = a + 1, c = a + nx + 1, d = c + 1;   /* 1-based */
            tris[3 * t] = a; tris[3 * t + 1] = b; tris[3 * t + 2] = d; ++t;
            tris[3 * t] = a; tris[3 * t + 1] = d; tris[3 * t + 2] = c; ++t;
        }
    const double mu = 3.2038120320e10, lam = mu;
    double *K = (double *)malloc(sizeof(double) * 6 * N * N);
    int rc = pq3d_assemble_dense_host(nodes, n_nodes, tris, N, mu, lam, 0, K, NULL);
    if (rc != PQ3D_OK) { fprintf(stderr, "assemble: %s\n", pq3d_last_error()); return 1; }
    /* the reference ABI at 3 points from one triangle */
    double X[3] = {500.0, 1500.0, -200.0}, Y[3] = {300.0, -700.0, 50.0}, Z[3] = {-1500.0, -2500.0, -800.0};
    double P1[3] = {0.0, 0.0, -1000.0}, P2[3] = {1000.0, 0.0, -1000.0}, P3[3] = {1000.0, 0.0, -2000.0};
    double stress[18], strain[18];
    TDstressFS_C(X, Y, Z, 3, P1, P2, P3, 1.0, 0.0, 0.0, mu, lam, false, stress, strain);
    /* an error is a status and a message, not an abort */
    const int bad = pq3d_assemble_dense_host(nodes, n_nodes, tris, 0, mu, lam, 0, K, NULL);
    const int bad_has_text = strlen(pq3d_last_error()) > 0;
    FILE *f = fopen(argv[1], "wb");
    if (!f) return 1;
    const int64_t hdr[4] = {N, n_nodes, bad, bad_has_text};
    fwrite(hdr, sizeof(int64_t), 4, f);
    fwrite(nodes, sizeof(double), 3 * n_nodes, f);
    fwrite(tris, sizeof(int64_t), 3 * N, f);
    fwrite(K, sizeof(double), 6 * N * N, f);
    fwrite(stress, sizeof(double), 18, f);
    fwrite(strain, sizeof(double), 18, f);
    fclose(f);
    printf("c host ok: N=%lld version %d\n", (long long)N, pq3d_version());
    free(nodes); free(tris); free(K);
    return 0;
}
