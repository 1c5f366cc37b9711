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

/* Read a whole snapshot from fp (XDR big-endian when standard != 0).
 * Returns 0, or -1 with a message in err (size errlen). */
int tipsy_read(FILE *fp, int standard, snapshot *s, char *err, size_t errlen);
void tipsy_free(snapshot *s);

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
