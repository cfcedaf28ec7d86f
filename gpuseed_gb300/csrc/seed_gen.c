/*
 * seed_gen.c -- drop-in for the reference's seed_gen executable.
 *
 *   seed_gen [-k INT] [-s] [-o] <index prefix> <reads.fa>
 *
 * Same options (getopt "k:so", seed_gen.cu:2826-2839), same index files and
 * the same stdout records (seed_gen.cu:3625-3647).  FASTA handling follows
 * the reference's getline loop (seed_gen.cu:2955-2990): lines starting with
 * '>' are skipped, every other line is one read whose last character (the
 * newline) is dropped.  Reads are processed in batches of at least -B bases
 * (64 Mi by default), numbered from 1 across batches; a reader thread parses
 * the next batch while the GPU seeds the current one and its records are
 * printed (formatted on the GPU).
 *
 * Extra options, off by default: -n (a non-ACGT base stops the extension),
 * -b (bwa's LF at row primary+1), -P (one-read-per-thread search kernel),
 * -B INT (bases per batch), -F (record-aware input: FASTA records over several
 * lines, FASTQ, CR LF line ends, a .gz file read through `gzip -dc`; a last
 * line without a newline keeps its last base), -c INT (drop seeds that occur
 * more than INT times, as bwa's -c), -T (build the text structures:
 * full suffix array, packed text and inverse-SA samples; they cost ~0.5 s of
 * load on 3.1 Gbp and pay off above a few hundred million reads), -Q (MEM
 * mode: a read's exclusion interval may come from the neighbouring read of
 * the batch, as seeds_to_threads_mem's scan finds it, seed_gen.cu:635-650;
 * batches then default to the reference's 1,000,000 bases, :2955, so that
 * the neighbours are the reference's).  Errors
 * print a message and exit with status 1, as the reference does for
 * unreadable index files.
 */
#define _GNU_SOURCE
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <pthread.h>
#include <unistd.h>

#include "../../include/gpuseed.h"

static double now_s(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return tv.tv_sec + tv.tv_usec * 1e-6;
}

/* -F: one record per call, sequence lines joined, CR stripped.  Returns the
 * sequence length, or -1 at end of input.  FASTQ records (header '@') are
 * four lines: header, sequence, '+', qualities. */
static ssize_t next_record(FILE *fp, char **line, size_t *line_cap, char **seq, size_t *seq_cap,
                           int *pending_header)
{
    size_t len = 0;
    int fastq = 0, have_header = *pending_header;
    ssize_t n;
    *pending_header = 0;
    for (;;) {
        n = getline(line, line_cap, fp);
        if (n < 0) break;
        while (n > 0 && ((*line)[n - 1] == '\n' || (*line)[n - 1] == '\r')) n--;
        if (n > 0 && ((*line)[0] == '>' || (*line)[0] == '@')) {
            if (have_header && len > 0) {
                *pending_header = 1;
                break;
            }
            if (have_header && !fastq && (*line)[0] == '>') { *pending_header = 1; break; }
            have_header = 1;
            fastq = (*line)[0] == '@';
            if (fastq) {
                ssize_t m = getline(line, line_cap, fp);
                if (m < 0) break;
                while (m > 0 && ((*line)[m - 1] == '\n' || (*line)[m - 1] == '\r')) m--;
                if (len + (size_t)m + 1 > *seq_cap) {
                    *seq_cap = 2 * (len + (size_t)m + 1);
                    *seq = (char *)realloc(*seq, *seq_cap);
                }
                memcpy(*seq + len, *line, (size_t)m);
                len += (size_t)m;
                if (getline(line, line_cap, fp) < 0 || getline(line, line_cap, fp) < 0) break;
                return (ssize_t)len;
            }
            continue;
        }
        if (len + (size_t)n + 1 > *seq_cap) {
            *seq_cap = 2 * (len + (size_t)n + 1);
            *seq = (char *)realloc(*seq, *seq_cap);
        }
        memcpy(*seq + len, *line, (size_t)n);
        len += (size_t)n;
        if (!have_header) return (ssize_t)len;   /* headerless: one line, one read */
    }
    if (n < 0 && len == 0 && !have_header) return -1;
    return (ssize_t)len;
}

static void die(const char *what, int rc)
{
    fprintf(stderr, "seed_gen: %s: %s (%s)\n", what, gs_strerror(rc), gs_last_error());
    exit(1);
}

/* One batch of reads as the reader thread fills it. */
typedef struct {
    char *bases;
    uint64_t *offs;
    uint32_t *lens;
    size_t cap_b, cap_r;
    uint64_t nb;
    uint32_t nr;
    int ready;   /* filled and waiting for the GPU */
    int last;    /* the input ends with this batch */
    int err;     /* out of host memory */
} batch_t;

/* The reader thread parses batch i+1 while the GPU seeds batch i and its
 * records are printed: two batches, handed back and forth. */
typedef struct {
    FILE *fp;
    int records;
    uint64_t batch_bases;
    batch_t b[2];
    pthread_mutex_t mu;
    pthread_cond_t cv;
    char *line, *rec;
    size_t line_cap, rec_cap;
    int pending_header;
    double t_load;
} reader_t;

static void fill_batch(reader_t *R, batch_t *B)
{
    B->nb = 0;
    B->nr = 0;
    B->last = 0;
    B->err = 0;
    while (B->nb < R->batch_bases) {
        const char *src;
        size_t L;
        if (R->records) {
            ssize_t n = next_record(R->fp, &R->line, &R->line_cap, &R->rec, &R->rec_cap,
                                    &R->pending_header);
            if (n < 0) {
                B->last = 1;
                break;
            }
            src = R->rec;
            L = (size_t)n;
        } else {
            ssize_t n = getline(&R->line, &R->line_cap, R->fp);
            if (n < 0) {
                B->last = 1;
                break;
            }
            if (R->line[0] == '>') continue;
            src = R->line;
            L = n > 0 ? (size_t)n - 1 : 0;
        }
        if (B->nb + L + 1 > B->cap_b) {
            size_t cap = B->cap_b ? B->cap_b : (1u << 20);
            while (B->nb + L + 1 > cap) cap *= 2;
            char *nbuf = (char *)realloc(B->bases, cap);
            if (!nbuf) {
                B->err = 1;
                return;
            }
            B->bases = nbuf;
            B->cap_b = cap;
        }
        if (B->nr + 1 > B->cap_r) {
            size_t cap = B->cap_r ? 2 * B->cap_r : (1u << 16);
            uint64_t *no = (uint64_t *)realloc(B->offs, cap * 8);
            if (no) B->offs = no;
            uint32_t *nl = (uint32_t *)realloc(B->lens, cap * 4);
            if (nl) B->lens = nl;
            if (!no || !nl) {
                B->err = 1;
                return;
            }
            B->cap_r = cap;
        }
        memcpy(B->bases + B->nb, src, L);
        B->offs[B->nr] = B->nb;
        B->lens[B->nr] = (uint32_t)L;
        B->nb += L;
        B->nr++;
    }
}

static void *reader_main(void *arg)
{
    reader_t *R = (reader_t *)arg;
    for (int i = 0;; i ^= 1) {
        batch_t *B = &R->b[i];
        pthread_mutex_lock(&R->mu);
        while (B->ready) pthread_cond_wait(&R->cv, &R->mu);
        pthread_mutex_unlock(&R->mu);
        double t0 = now_s();
        fill_batch(R, B);
        R->t_load += now_s() - t0;
        int stop = B->last || B->err;
        pthread_mutex_lock(&R->mu);
        B->ready = 1;
        pthread_cond_broadcast(&R->cv);
        pthread_mutex_unlock(&R->mu);
        if (stop) break;
    }
    return NULL;
}

int main(int argc, char *argv[])
{
    double t_start = now_s();
    gs_params p;
    memset(&p, 0, sizeof(p));
    p.k = 20;
    uint64_t batch_bases = 64u << 20;
    int print_out = 0, records = 0, text = 0, batch_set = 0, c;
    while ((c = getopt(argc, argv, "k:sonbPB:Fc:TQ")) >= 0) {
        switch (c) {
        case 'k': p.k = atoi(optarg); break;
        case 's': p.smem = 1; break;
        case 'o': print_out = 1; break;
        case 'n': p.n_mode = GS_N_STOP; break;
        case 'b': p.lf_mode = GS_LF_BWA; break;
        case 'P': p.kernel = GS_KERNEL_PLAIN; break;
        case 'B': batch_bases = strtoull(optarg, NULL, 10); batch_set = 1; break;
        case 'F': records = 1; break;
        case 'c': p.max_occ = atoi(optarg); break;
        case 'T': text = 1; break;
        case 'Q': p.mem_next = GS_MEM_NEXT_GPUSEED; break;
        default: break;
        }
    }
    if (p.mem_next && !batch_set) batch_bases = 1000000;
    if (optind + 2 > argc) {
        fprintf(stderr, "Usage: seed_gen [-k <minimum seed length>] [-s] [-o] <index prefix> "
                        "<reads fasta file>\n");
        return 1;
    }
    if (batch_bases == 0) batch_bases = 1;
    fprintf(stderr, "Loading index from file and copying it to GPU...\n");
    double t0 = now_s();
    gs_index *idx = NULL;
    int rc = gs_index_load(argv[optind], 0, &idx);
    if (rc) die("loading index", rc);
    if (text && (rc = gs_index_set_text(idx, 4)) != GS_OK) die("building the text structures", rc);
    gs_index_info info;
    gs_index_get_info(idx, &info);
    fprintf(stderr, "seq_len=%u primary=%u sa_intv=%u; index and 13-mer table on GPU in %.3f s\n",
            info.seq_len, info.primary, info.sa_intv, now_s() - t0);
    gs_ctx *ctx = NULL;
    rc = gs_ctx_create(idx, NULL, &ctx);
    if (rc) die("creating context", rc);

    const char *fname = argv[optind + 1];
    size_t fl = strlen(fname);
    int piped = records && fl > 3 && strcmp(fname + fl - 3, ".gz") == 0;
    FILE *fp;
    if (piped) {
        char *cmd = (char *)malloc(fl + 32);
        snprintf(cmd, fl + 32, "gzip -dc -- '%s'", fname);
        fp = popen(cmd, "r");
        free(cmd);
    } else {
        fp = fopen(fname, "r");
    }
    if (!fp) {
        fprintf(stderr, "seed_gen: cannot open %s\n", argv[optind + 1]);
        return 1;
    }
    reader_t R;
    memset(&R, 0, sizeof(R));
    R.fp = fp;
    R.records = records;
    R.batch_bases = batch_bases;
    pthread_mutex_init(&R.mu, NULL);
    pthread_cond_init(&R.cv, NULL);
    pthread_t reader;
    if (pthread_create(&reader, NULL, reader_main, &R) != 0) {
        fprintf(stderr, "seed_gen: cannot start the reader thread\n");
        return 1;
    }
    uint32_t reads_done = 0;
    double t_gpu = 0, t_print = 0;
    for (int i = 0;; i ^= 1) {
        batch_t *B = &R.b[i];
        pthread_mutex_lock(&R.mu);
        while (!B->ready) pthread_cond_wait(&R.cv, &R.mu);
        pthread_mutex_unlock(&R.mu);
        if (B->err) {
            fprintf(stderr, "seed_gen: out of host memory\n");
            return 1;
        }
        const int last = B->last;
        if (B->nr) {
            double tg = now_s();
            rc = gs_seed(ctx, B->bases, B->offs, B->lens, B->nr, &p);
            if (rc) die("seeding batch", rc);
            t_gpu += now_s() - tg;
            gs_result_view v;
            gs_result_host(ctx, &v);
            fprintf(stderr, "batch of %u reads: %llu seeds, %llu positions, %.3f s on GPU\n", B->nr,
                    (unsigned long long)v.n_seeds, (unsigned long long)v.n_pos, now_s() - tg);
            if (print_out) {
                double tp = now_s();
                fflush(stdout);
                rc = gs_result_write_text(ctx, 1, reads_done + 1, p.smem);
                if (rc) die("writing records", rc);
                t_print += now_s() - tp;
            }
            reads_done += B->nr;
        }
        pthread_mutex_lock(&R.mu);
        B->ready = 0;
        pthread_cond_broadcast(&R.cv);
        pthread_mutex_unlock(&R.mu);
        if (last) break;
    }
    pthread_join(reader, NULL);
    if (piped) pclose(fp);
    else fclose(fp);
    free(R.line);
    free(R.rec);
    for (int i = 0; i < 2; i++) {
        free(R.b[i].bases);
        free(R.b[i].offs);
        free(R.b[i].lens);
    }
    gs_ctx_free(ctx);
    gs_index_free(idx);
    fprintf(stderr,
            "%s seeds: %u reads, GPU time %.3f s, load %.3f s (overlapped), print %.3f s, total "
            "%.3f s\n",
            p.smem ? "SMEM" : "MEM", reads_done, t_gpu, R.t_load, t_print, now_s() - t_start);
    return 0;
}
