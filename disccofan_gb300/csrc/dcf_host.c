/*
 * Host-side C helpers of the C ABI that need no GPU: lambda vectors and FITS input.
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

/*
 * dcf_fits_read: the primary image of a FITS file as the reference's FITS input
 * (io.c:624-706 through CFITSIO's fits_read_pix into float) sees it: every pixel
 * BZERO + BSCALE * raw, stored as float, x fastest, rows in file order.  The
 * header is a run of 2880-byte blocks of 80-character "KEY     = value" cards
 * ending with END; the data follow big-endian.  BITPIX 8 (unsigned), 16, 32
 * (signed), -32 and -64 (IEEE) are read; NAXIS must be 1 to 3.
 */
static int card_int(const char *card, long long *v)
{
    char *end;
    *v = strtoll(card + 10, &end, 10);
    return end != card + 10;
}

static int card_double(const char *card, double *v)
{
    char buf[71];
    memcpy(buf, card + 10, 70);
    buf[70] = 0;
    for (char *p = buf; *p; p++)
        if (*p == 'D') *p = 'E';  /* Fortran exponent */
    char *end;
    *v = strtod(buf, &end);
    return end != buf;
}

static double be_value(const unsigned char *p, int bitpix)
{
    switch (bitpix) {
    case 8: return (double)p[0];
    case 16: {
        unsigned u = ((unsigned)p[0] << 8) | p[1];
        return (double)(short)(unsigned short)u;
    }
    case 32: {
        unsigned u = ((unsigned)p[0] << 24) | ((unsigned)p[1] << 16) | ((unsigned)p[2] << 8) | p[3];
        return (double)(int)u;
    }
    case -32: {
        unsigned u = ((unsigned)p[0] << 24) | ((unsigned)p[1] << 16) | ((unsigned)p[2] << 8) | p[3];
        float f;
        memcpy(&f, &u, 4);
        return (double)f;
    }
    default: {
        unsigned long long u = 0;
        for (int i = 0; i < 8; i++) u = (u << 8) | p[i];
        double d;
        memcpy(&d, &u, 8);
        return d;
    }
    }
}

/* Header of the primary HDU: BITPIX, axis lengths (1 for missing axes), BZERO and
 * BSCALE; the file is left at the first data byte. */
static dcf_status fits_header(FILE *f, long long *bp, uint64_t dims[3], double *bzero, double *bscale)
{
    char block[2880];
    long long naxis = -1, ax[3] = {1, 1, 1};
    int have_bitpix = 0, done = 0;
    *bzero = 0.0;
    *bscale = 1.0;
    while (!done) {
        if (fread(block, 1, 2880, f) != 2880) return DCF_ERR_IO;
        for (int k = 0; k < 36 && !done; k++) {
            const char *card = block + 80 * k;
            if (!strncmp(card, "END     ", 8)) {
                done = 1;
            } else if (card[8] == '=' && card[9] == ' ') {
                if (!strncmp(card, "BITPIX  ", 8)) have_bitpix = card_int(card, bp);
                else if (!strncmp(card, "NAXIS   ", 8)) card_int(card, &naxis);
                else if (!strncmp(card, "NAXIS1  ", 8)) card_int(card, &ax[0]);
                else if (!strncmp(card, "NAXIS2  ", 8)) card_int(card, &ax[1]);
                else if (!strncmp(card, "NAXIS3  ", 8)) card_int(card, &ax[2]);
                else if (!strncmp(card, "BZERO   ", 8)) card_double(card, bzero);
                else if (!strncmp(card, "BSCALE  ", 8)) card_double(card, bscale);
            }
        }
    }
    if (!have_bitpix || (*bp != 8 && *bp != 16 && *bp != 32 && *bp != -32 && *bp != -64) || naxis < 1 ||
        naxis > 3 || ax[0] < 1 || ax[1] < 1 || ax[2] < 1)
        return DCF_ERR_UNSUPPORTED;
    for (int i = 0; i < 3; i++) dims[i] = (uint64_t)(i < naxis ? ax[i] : 1);
    return DCF_OK;
}

dcf_status dcf_fits_read(const char *path, float *out, uint64_t capacity, uint64_t dims[3], int *bitpix)
{
    if (!path || !dims) return DCF_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return DCF_ERR_IO;
    long long bp = 0;
    double bzero, bscale;
    dcf_status st = fits_header(f, &bp, dims, &bzero, &bscale);
    if (st != DCF_OK) {
        fclose(f);
        return st;
    }
    if (bitpix) *bitpix = (int)bp;
    const uint64_t n = dims[0] * dims[1] * dims[2];
    if (!out) {
        fclose(f);
        return DCF_OK;
    }
    if (capacity < n) {
        fclose(f);
        return DCF_ERR_INVALID;
    }
    const int bytes = (int)(bp < 0 ? -bp : bp) / 8;
    unsigned char buf[8 * 4096];
    uint64_t done_px = 0;
    while (done_px < n) {
        uint64_t chunk = n - done_px < 4096 ? n - done_px : 4096;
        if (fread(buf, (size_t)bytes, chunk, f) != chunk) {
            fclose(f);
            return DCF_ERR_IO;
        }
        for (uint64_t i = 0; i < chunk; i++) out[done_px + i] = (float)(bzero + bscale * be_value(buf + i * bytes, (int)bp));
        done_px += chunk;
    }
    fclose(f);
    return DCF_OK;
}

/*
 * dcf_fits_read_raw: the same image in its own pixel type, for the tree build to
 * take without a float copy on the host: BITPIX 8 (BZERO 0) as u8, BITPIX 16 with
 * BZERO 32768 (FITS's unsigned 16-bit convention) as u16, BITPIX 32 with BZERO
 * 2147483648 as u32, BITPIX -32 as f32; BSCALE must be 1.  Converted to float the
 * values equal dcf_fits_read's (the build converts u32 with the same rounding).
 */
dcf_status dcf_fits_read_raw(const char *path, void *out, uint64_t capacity_bytes, uint64_t dims[3], int *dtype)
{
    if (!path || !dims || !dtype) return DCF_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return DCF_ERR_IO;
    long long bp = 0;
    double bzero, bscale;
    dcf_status st = fits_header(f, &bp, dims, &bzero, &bscale);
    if (st == DCF_OK) {
        if (bscale != 1.0) st = DCF_ERR_UNSUPPORTED;
        else if (bp == 8 && bzero == 0.0) *dtype = DCF_U8;
        else if (bp == 16 && bzero == 32768.0) *dtype = DCF_U16;
        else if (bp == 32 && bzero == 2147483648.0) *dtype = DCF_U32;
        else if (bp == -32 && bzero == 0.0) *dtype = DCF_F32;
        else st = DCF_ERR_UNSUPPORTED;
    }
    if (st != DCF_OK || !out) {
        fclose(f);
        return st;
    }
    const int bytes = (int)(bp < 0 ? -bp : bp) / 8;
    const uint64_t n = dims[0] * dims[1] * dims[2];
    if (capacity_bytes / (uint64_t)bytes < n) {
        fclose(f);
        return DCF_ERR_INVALID;
    }
    unsigned char *o = (unsigned char *)out;
    if (fread(o, (size_t)bytes, (size_t)n, f) != (size_t)n) {
        fclose(f);
        return DCF_ERR_IO;
    }
    fclose(f);
    /* big-endian to host order; the offset BZERO of the unsigned types flips the top bit */
    for (uint64_t i = 0; i < n; i++) {
        unsigned char *p = o + i * (uint64_t)bytes;
        if (bytes == 2) {
            const uint16_t v = (uint16_t)((((unsigned)p[0] << 8) | p[1]) ^ 0x8000u);
            memcpy(p, &v, 2);
        } else if (bytes == 4) {
            uint32_t v = ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
            if (bp == 32) v ^= 0x80000000u;
            memcpy(p, &v, 4);
        }
    }
    return DCF_OK;
}
