/*
 * TIPSY input and skid output files (see tipsy_io.h).
 */
#include "tipsy_io.h"

#include "skid_gpu.h"

#include <errno.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define GAS_FLOATS 12
#define DARK_FLOATS 9
#define STAR_FLOATS 11

static uint32_t bswap32(uint32_t v)
{
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}

static int host_is_little(void)
{
    uint32_t one = 1;
    return *(unsigned char *)&one == 1;
}

/* Read count 4-byte words (floats or ints); XDR words are big-endian. */
static int read_words(FILE *fp, void *dst, size_t count, int big)
{
    if (fread(dst, 4, count, fp) != count) return -1;
    if (big == host_is_little()) {
        uint32_t *w = (uint32_t *)dst;
        for (size_t i = 0; i < count; ++i) w[i] = bswap32(w[i]);
    }
    return 0;
}

static int write_words(FILE *fp, const void *src, size_t count, int big)
{
    if (big != host_is_little()) return fwrite(src, 4, count, fp) == count ? 0 : -1;
    const uint32_t *w = (const uint32_t *)src;
    for (size_t i = 0; i < count; ++i) {
        uint32_t v = bswap32(w[i]);
        if (fwrite(&v, 4, 1, fp) != 1) return -1;
    }
    return 0;
}

static int read_header(FILE *fp, int standard, double *time, int cnt[5])
{
    unsigned char raw[32];
    if (fread(raw, 1, 32, fp) != 32) return -1;
    uint64_t t;
    memcpy(&t, raw, 8);
    if (standard == host_is_little()) {
        uint64_t r = 0;
        for (int i = 0; i < 8; ++i) r = (r << 8) | ((t >> (8 * i)) & 0xff);
        t = r;
    }
    memcpy(time, &t, 8);
    for (int i = 0; i < 5; ++i) {
        uint32_t v;
        memcpy(&v, raw + 8 + 4 * i, 4);
        if (standard == host_is_little()) v = bswap32(v);
        cnt[i] = (int)v;
    }
    return 0;
}

static int write_header(FILE *fp, int standard, double time, int nbodies, int nsph, int ndark,
                        int nstar)
{
    unsigned char raw[32];
    memset(raw, 0, sizeof(raw));
    uint64_t t;
    memcpy(&t, &time, 8);
    if (standard == host_is_little()) {
        uint64_t r = 0;
        for (int i = 0; i < 8; ++i) r = (r << 8) | ((t >> (8 * i)) & 0xff);
        t = r;
    }
    memcpy(raw, &t, 8);
    int v[6] = {nbodies, 3, nsph, ndark, nstar, 0};
    for (int i = 0; i < 6; ++i) {
        uint32_t w = (uint32_t)v[i];
        if (standard == host_is_little()) w = bswap32(w);
        memcpy(raw + 8 + 4 * i, &w, 4);
    }
    return fwrite(raw, 1, 32, fp) == 32 ? 0 : -1;
}

int tipsy_read_raw(FILE *fp, int standard, tipsy_raw *r, char *err, size_t errlen)
{
    memset(r, 0, sizeof(*r));
    int cnt[5];
    if (read_header(fp, standard, &r->time, cnt)) {
        snprintf(err, errlen, "truncated TIPSY header");
        return -1;
    }
    r->nGas = cnt[2];
    r->nDark = cnt[3];
    r->nStar = cnt[4];
    if (r->nGas < 0 || r->nDark < 0 || r->nStar < 0 ||
        (long long)r->nGas + r->nDark + r->nStar > (1ll << 28)) {
        snprintf(err, errlen, "bad particle counts in TIPSY header (%d gas, %d dark, %d star)",
                 r->nGas, r->nDark, r->nStar);
        return -1;
    }
    r->n = r->nGas + r->nDark + r->nStar;
    r->bytes = 4 * ((size_t)GAS_FLOATS * r->nGas + (size_t)DARK_FLOATS * r->nDark +
                    (size_t)STAR_FLOATS * r->nStar);
    size_t m = r->bytes ? r->bytes : 4;
    if (skid_host_alloc(m, &r->records) == SKID_OK) {
        r->pinned = 1;
    } else {
        r->records = malloc(m);
        r->pinned = 0;
    }
    if (!r->records) {
        snprintf(err, errlen, "out of host memory");
        return -1;
    }
    if (fread(r->records, 1, r->bytes, fp) != r->bytes) {
        snprintf(err, errlen, "truncated TIPSY particle records");
        tipsy_raw_free(r);
        return -1;
    }
    return 0;
}

void tipsy_raw_free(tipsy_raw *r)
{
    if (r->pinned)
        skid_host_free(r->records);
    else
        free(r->records);
    memset(r, 0, sizeof(*r));
}

void tipsy_raw_positions(const tipsy_raw *r, int standard, float *pos)
{
    const unsigned char *b = r->records;
    const int swap = standard == host_is_little();
    for (int i = 0; i < r->n; ++i) {
        size_t off = i < r->nGas ? 4 * (size_t)GAS_FLOATS * i
                     : i < r->nGas + r->nDark
                         ? 4 * ((size_t)GAS_FLOATS * r->nGas + (size_t)DARK_FLOATS * (i - r->nGas))
                         : 4 * ((size_t)GAS_FLOATS * r->nGas + (size_t)DARK_FLOATS * r->nDark +
                                (size_t)STAR_FLOATS * (i - r->nGas - r->nDark));
        for (int d = 0; d < 3; ++d) {
            uint32_t w;
            memcpy(&w, b + off + 4 * (1 + d), 4);
            if (swap) w = bswap32(w);
            memcpy(&pos[3 * (size_t)i + d], &w, 4);
        }
    }
}

void tipsy_free(snapshot *s)
{
    free(s->pos);
    free(s->vel);
    free(s->mass);
    free(s->soft);
    free(s->temp);
    memset(s, 0, sizeof(*s));
}

int tipsy_write_gtp(const char *path, int standard, double time, int nGroup, const float *mass,
                    const float *pos, const float *vel, const float *radius)
{
    FILE *fp = fopen(path, "wb");
    if (!fp) return -1;
    int rc = write_header(fp, standard, time, nGroup, 0, 0, nGroup);
    for (int g = 0; g < nGroup && !rc; ++g) {
        float rec[STAR_FLOATS];
        rec[0] = mass[g];
        for (int d = 0; d < 3; ++d) {
            rec[1 + d] = pos[3 * (size_t)g + d];
            rec[4 + d] = vel[3 * (size_t)g + d];
        }
        rec[7] = 0.0f;           /* metals */
        rec[8] = (float)time;    /* tform */
        rec[9] = radius[g];      /* eps */
        rec[10] = 0.0f;          /* phi */
        rc = write_words(fp, rec, STAR_FLOATS, standard);
    }
    if (fclose(fp)) rc = -1;
    return rc;
}

int tipsy_read_gtp(const char *path, int standard, int *nStar, float **mass, float **pos,
                   float **vel, char *err, size_t errlen)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) return 0;
    double t;
    int cnt[5];
    if (read_header(fp, standard, &t, cnt) || cnt[2] < 0 || cnt[3] < 0 || cnt[4] < 0) {
        snprintf(err, errlen, "%s: bad TIPSY header", path);
        fclose(fp);
        return -1;
    }
    /* skip gas and dark records (kd.c:1121-1128) */
    if (fseek(fp, (long)cnt[2] * GAS_FLOATS * 4 + (long)cnt[3] * DARK_FLOATS * 4, SEEK_CUR)) {
        snprintf(err, errlen, "%s: truncated", path);
        fclose(fp);
        return -1;
    }
    int ns = cnt[4];
    size_t m = ns > 0 ? (size_t)ns : 1;
    *mass = malloc(m * sizeof(float));
    *pos = malloc(3 * m * sizeof(float));
    *vel = malloc(3 * m * sizeof(float));
    for (int i = 0; i < ns; ++i) {
        float rec[STAR_FLOATS];
        if (read_words(fp, rec, STAR_FLOATS, standard)) {
            snprintf(err, errlen, "%s: truncated star records", path);
            fclose(fp);
            return -1;
        }
        (*mass)[i] = rec[0];
        for (int d = 0; d < 3; ++d) {
            (*pos)[3 * (size_t)i + d] = rec[1 + d];
            (*vel)[3 * (size_t)i + d] = rec[4 + d];
        }
    }
    fclose(fp);
    *nStar = ns;
    return 1;
}

/* Fast decimal output for the large text files. */
static char *put_int(char *p, int v)
{
    char tmp[16];
    int k = 0;
    unsigned u = v < 0 ? (unsigned)(-(long long)v) : (unsigned)v;
    if (v < 0) *p++ = '-';
    do { tmp[k++] = (char)('0' + u % 10); u /= 10; } while (u);
    while (k) *p++ = tmp[--k];
    *p++ = '\n';
    return p;
}

/* One line per value, formatted in parallel chunks on the host's cores and
 * written in order: the same bytes as formatting the lines one after
 * another.  fmt writes line i at p (at most maxlen bytes, plus a NUL it may
 * leave after them) and returns its length. */
typedef size_t (*line_fmt)(char *p, const void *data, size_t i);

typedef struct {
    line_fmt fmt;
    const void *data;
    size_t lo, hi, len;
    char *buf;
} line_job;

static void *format_lines(void *arg)
{
    line_job *j = (line_job *)arg;
    char *p = j->buf;
    for (size_t i = j->lo; i < j->hi; ++i) p += j->fmt(p, j->data, i);
    j->len = (size_t)(p - j->buf);
    return NULL;
}

enum { LINE_THREADS_MAX = 16 };
/* Lines formatted per block (bounds the text held at once). */
#define LINE_BLOCK ((size_t)1 << 22)

/* Lines [lo, hi) in nt chunks, then written in order. */
static int write_block(FILE *fp, size_t lo, size_t hi, int nt, line_fmt fmt, const void *data,
                       size_t maxlen)
{
    line_job job[LINE_THREADS_MAX];
    pthread_t th[LINE_THREADS_MAX];
    int started[LINE_THREADS_MAX] = {0};
    const size_t n = hi - lo, per = (n + (size_t)nt - 1) / (size_t)nt;
    int rc = 0;
    for (int t = 0; t < nt; ++t) {
        job[t].fmt = fmt;
        job[t].data = data;
        job[t].lo = lo + ((size_t)t * per < n ? (size_t)t * per : n);
        job[t].hi = lo + ((size_t)(t + 1) * per < n ? (size_t)(t + 1) * per : n);
        job[t].len = 0;
        job[t].buf = malloc((job[t].hi - job[t].lo) * maxlen + 1);
        if (!job[t].buf) rc = -1;
    }
    if (!rc) {
        for (int t = 1; t < nt; ++t)
            started[t] = pthread_create(&th[t], NULL, format_lines, &job[t]) == 0;
        format_lines(&job[0]);
        for (int t = 1; t < nt; ++t) {
            if (started[t]) pthread_join(th[t], NULL);
            else format_lines(&job[t]);   /* no thread: this one formats the chunk */
        }
        for (int t = 0; t < nt && !rc; ++t)
            if (fwrite(job[t].buf, 1, job[t].len, fp) != job[t].len) rc = -1;
    }
    for (int t = 0; t < nt; ++t) free(job[t].buf);
    return rc;
}

static int write_lines(FILE *fp, size_t n, line_fmt fmt, const void *data, size_t maxlen)
{
    int nt = 1;
    if (n >= 65536) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        nt = c < 1 ? 1 : c > LINE_THREADS_MAX ? LINE_THREADS_MAX : (int)c;
    }
    int rc = 0;
    for (size_t lo = 0; lo < n && !rc; lo += LINE_BLOCK)
        rc = write_block(fp, lo, lo + LINE_BLOCK < n ? lo + LINE_BLOCK : n, nt, fmt, data, maxlen);
    return rc;
}

static size_t grp_line(char *p, const void *data, size_t i)
{
    return (size_t)(put_int(p, ((const int *)data)[i]) - p);
}

int write_grp(const char *path, int n, const int *grp)
{
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    char head[16];
    int rc = fwrite(head, 1, (size_t)(put_int(head, n) - head), fp) ? 0 : -1;
    if (!rc && n > 0) rc = write_lines(fp, (size_t)n, grp_line, grp, 12);
    return fclose(fp) || rc ? -1 : 0;
}

static size_t den_line(char *p, const void *data, size_t i)
{
    return (size_t)snprintf(p, 32, "%.10g\n", ((const float *)data)[i]);
}

int write_den(const char *path, int n, const float *rho)
{
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    int rc = fprintf(fp, "%d\n", n) < 0 ? -1 : 0;
    if (!rc && n > 0) rc = write_lines(fp, (size_t)n, den_line, rho, 31);
    return fclose(fp) || rc ? -1 : 0;
}

typedef struct {
    const snapshot *s;
    const float *moved;
    const int *flag;
    float h[3];
} ray_data;

/* Line d*n + i: the wrapped displacement of particle i along axis d. */
static size_t ray_line(char *p, const void *data, size_t k)
{
    const ray_data *r = (const ray_data *)data;
    const size_t n = (size_t)r->s->n, i = k % n;
    const int d = (int)(k / n);
    if (!r->flag[i]) {
        p[0] = '0';
        p[1] = '\n';
        return 2;
    }
    float dx = r->moved[3 * i + d] - r->s->pos[3 * i + d];
    const float h = r->h[d];
    if (dx > h) dx -= 2 * h;
    if (dx <= -h) dx += 2 * h;
    return (size_t)snprintf(p, 32, "%g\n", dx);
}

int write_ray(const char *path, const snapshot *s, const float *moved, const int *moved_flag,
              const float period[3])
{
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    int rc = fprintf(fp, "%d\n", s->n) < 0 ? -1 : 0;
    ray_data r = {s, moved, moved_flag, {0.0f, 0.0f, 0.0f}};
    for (int d = 0; d < 3; ++d) r.h[d] = (float)(0.5 * (double)period[d]);
    if (!rc && s->n > 0) rc = write_lines(fp, 3 * (size_t)s->n, ray_line, &r, 31);
    return fclose(fp) || rc ? -1 : 0;
}

int read_grp(const char *path, int **grp, char *err, size_t errlen)
{
    FILE *fp = fopen(path, "r");
    if (!fp) {
        snprintf(err, errlen, "ERROR: Could not open file:%s", path);
        return -1;
    }
    int n = 0;
    if (fscanf(fp, "%d", &n) != 1 || n < 0) {
        snprintf(err, errlen, "%s: bad particle count", path);
        fclose(fp);
        return -1;
    }
    *grp = malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    for (int i = 0; i < n; ++i) {
        if (fscanf(fp, "%d", &(*grp)[i]) != 1) {
            snprintf(err, errlen, "%s: truncated after %d of %d ids", path, i, n);
            fclose(fp);
            return -1;
        }
    }
    fclose(fp);
    return n;
}
