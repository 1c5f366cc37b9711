/*
 * Big-endian XDR primitives over a stdio FILE (RFC 4506 section 4.1, 4.6,
 * 4.7).  Project-written replacement for the SunRPC/tirpc routines that the
 * reference skid's TIPSY "-std" reader and writer call.  Test infrastructure
 * only: used to build the reference for the oracle, never linked into the
 * product library.
 */
#include <stdint.h>
#include <string.h>
#include "rpc/xdr.h"

void xdrstdio_create(XDR *xdrs, FILE *fp, enum xdr_op op)
{
    xdrs->x_op = op;
    xdrs->fp = fp;
}

void xdr_destroy(XDR *xdrs)
{
    if (xdrs->x_op == XDR_ENCODE && xdrs->fp) fflush(xdrs->fp);
    xdrs->fp = NULL;
}

static bool_t put_be(XDR *xdrs, uint64_t v, int nbytes)
{
    unsigned char b[8];
    for (int i = 0; i < nbytes; ++i) b[i] = (unsigned char)(v >> (8 * (nbytes - 1 - i)));
    return fwrite(b, 1, (size_t)nbytes, xdrs->fp) == (size_t)nbytes;
}

static bool_t get_be(XDR *xdrs, uint64_t *v, int nbytes)
{
    unsigned char b[8];
    if (fread(b, 1, (size_t)nbytes, xdrs->fp) != (size_t)nbytes) return FALSE;
    uint64_t r = 0;
    for (int i = 0; i < nbytes; ++i) r = (r << 8) | b[i];
    *v = r;
    return TRUE;
}

static bool_t xdr_word(XDR *xdrs, void *p, int nbytes)
{
    uint64_t v = 0;
    if (xdrs->x_op == XDR_ENCODE) {
        if (nbytes == 4) { uint32_t w; memcpy(&w, p, 4); v = w; }
        else memcpy(&v, p, 8);
        return put_be(xdrs, v, nbytes);
    }
    if (xdrs->x_op == XDR_DECODE) {
        if (!get_be(xdrs, &v, nbytes)) return FALSE;
        if (nbytes == 4) { uint32_t w = (uint32_t)v; memcpy(p, &w, 4); }
        else memcpy(p, &v, 8);
        return TRUE;
    }
    return TRUE;
}

bool_t xdr_int(XDR *xdrs, int *ip) { return xdr_word(xdrs, ip, 4); }
bool_t xdr_float(XDR *xdrs, float *fp) { return xdr_word(xdrs, fp, 4); }
bool_t xdr_double(XDR *xdrs, double *dp) { return xdr_word(xdrs, dp, 8); }

bool_t xdr_vector(XDR *xdrs, char *base, unsigned int nelem,
                  unsigned int elsize, xdrproc_t proc)
{
    for (unsigned int i = 0; i < nelem; ++i) {
        if (!proc(xdrs, base + (size_t)i * elsize)) return FALSE;
    }
    return TRUE;
}
