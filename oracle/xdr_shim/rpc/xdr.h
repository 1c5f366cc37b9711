/*
 * Minimal stand-in for <rpc/xdr.h> (RFC 4506 external data representation),
 * written for this project.  XDR stores 32-bit ints and floats as big-endian
 * 4-byte words and doubles as big-endian 8-byte words.  Only the stdio stream
 * and the primitives used by skid's TIPSY reader/writer are provided.
 */
#ifndef SKID_SHIM_RPC_XDR_H
#define SKID_SHIM_RPC_XDR_H

#include <stdio.h>
#include "types.h"

enum xdr_op { XDR_ENCODE = 0, XDR_DECODE = 1, XDR_FREE = 2 };

typedef struct XDR {
    enum xdr_op x_op;
    FILE *fp;
} XDR;

typedef bool_t (*xdrproc_t)(XDR *, void *, ...);

void xdrstdio_create(XDR *xdrs, FILE *fp, enum xdr_op op);
void xdr_destroy(XDR *xdrs);
bool_t xdr_int(XDR *xdrs, int *ip);
bool_t xdr_float(XDR *xdrs, float *fp);
bool_t xdr_double(XDR *xdrs, double *dp);
bool_t xdr_vector(XDR *xdrs, char *base, unsigned int nelem,
                  unsigned int elsize, xdrproc_t proc);

#endif
