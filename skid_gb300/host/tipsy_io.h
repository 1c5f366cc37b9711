/*
 * TIPSY snapshot input and skid's output files, host side of the `skid` CLI.
 *
 * Formats follow the reference: header struct dump (tipsydefs.h:39-46; 32
 * bytes native, explicit pad word in XDR, kd.c:16-28), gas/dark/star records
 * of 12/9/11 floats read in that order (kd.c:164-217), .grp/.den/.ray text
 * (kd.c:1502-1608), .gtp star records (kd.c:1611-1687).
 */
#ifndef SKID_TIPSY_IO_H
#define SKID_TIPSY_IO_H

#include <stdio.h>

typedef struct snapshot {
    double time;
    int nGas, nDark, nStar, n;
    float *pos, *vel;      /* 3n, iOrder */
    float *mass, *soft, *temp;
} snapshot;

/* Frees the arrays a snapshot holds (NULL ones included). */
void tipsy_free(snapshot *s);

/* The header and the particle records as they lie in the file (XDR
 * big-endian when standard != 0), for skid_set_tipsy: one fread of the
 * whole record block into page-locked memory (skid_host_alloc; plain malloc
 * where that is unavailable).  Returns 0, or -1 with a message in err. */
typedef struct tipsy_raw {
    double time;
    int nGas, nDark, nStar, n;
    void *records;
    size_t bytes;
    int pinned;
} tipsy_raw;
int tipsy_read_raw(FILE *fp, int standard, tipsy_raw *r, char *err, size_t errlen);
void tipsy_raw_free(tipsy_raw *r);
/* Decode the positions (3n floats, iOrder) of the raw records on the host. */
void tipsy_raw_positions(const tipsy_raw *r, int standard, float *pos);

/* .gtp: nGroup star records (mass, pos, vel, eps=radius, tform=time). */
int tipsy_write_gtp(const char *path, int standard, double time, int nGroup,
                    const float *mass, const float *pos, const float *vel,
                    const float *radius);

/* Star records of a .gtp file for unbind-only mode (kd.c:1083-1160): fills
 * pos/vel (3*nStar each, caller frees) and *nStar; returns 1 if the file
 * was read, 0 if it does not exist, -1 on a malformed file. */
int tipsy_read_gtp(const char *path, int standard, int *nStar, float **mass, float **pos,
                   float **vel, char *err, size_t errlen);

int write_grp(const char *path, int n, const int *grp);
int write_den(const char *path, int n, const float *rho);
int write_ray(const char *path, const snapshot *s, const float *moved, const int *moved_flag,
              const float period[3]);
/* Reads N then N group ids; returns N or -1. */
int read_grp(const char *path, int **grp, char *err, size_t errlen);

#endif
