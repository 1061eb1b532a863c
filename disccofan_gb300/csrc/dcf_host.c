/*
 * Host-side C helpers of the C ABI that need no GPU.
 *
 * dcf_lvec_read restates lambda_vector_read (lambdavec.c:35-84): the first line of
 * the file is the "#LambdaVector file..." header, then whitespace-separated float
 * values.  The result has one more entry than the file: out[0] = 0, then each value
 * divided by imscale (computed in double, stored as float, as the reference's
 * `l->lambdas[c+1] /= im_scale` does).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/dcf.h"

dcf_status dcf_lvec_read(const char *path, double imscale, float *out, int capacity, int *num_lambdas)
{
    if (!path || !num_lambdas) return DCF_ERR_INVALID;
    if (imscale == 0.0) return DCF_ERR_INVALID;
    FILE *f = fopen(path, "r");
    if (!f) return DCF_ERR_IO;
    char line[512];
    if (!fgets(line, sizeof line, f) || line[0] != '#') {
        fclose(f);
        return DCF_ERR_IO;
    }
    int count = 0;
    float v;
    long start = ftell(f);
    while (fscanf(f, "%f", &v) == 1) count++;
    *num_lambdas = count + 1;
    if (!out) {
        fclose(f);
        return DCF_OK;
    }
    if (capacity < count + 1) {
        fclose(f);
        return DCF_ERR_INVALID;
    }
    fseek(f, start, SEEK_SET);
    out[0] = 0.0f;
    for (int c = 0; c < count; c++) {
        if (fscanf(f, "%f", &v) != 1) {
            fclose(f);
            return DCF_ERR_IO;
        }
        out[c + 1] = (float)((double)v / imscale);
    }
    fclose(f);
    return DCF_OK;
}
