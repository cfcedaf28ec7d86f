/*
 * gpuseed_synth.h -- seeded synthetic references and reads.
 *
 * The reference publishes no dataset and no benchmark inputs; these
 * generators stand in for the workloads it is quoted on (uniform or
 * GC-biased background, segmental duplications, diverged repeat families, N
 * blocks; reads from both strands with substitutions, short indels and N
 * runs).  Integer-only random draws (splitmix64 / xoshiro256**), so a spec
 * and seed give the same bytes on every machine.
 */
#ifndef GPUSEED_SYNTH_H
#define GPUSEED_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint64_t length;
    uint64_t seed;
    double gc;                       /* G+C fraction of the background */
    double dup_frac;                 /* fraction of bases written by duplicated segments */
    uint32_t dup_len_min, dup_len_max;
    double dup_div_min, dup_div_max; /* per-copy substitution rate */
    uint32_t fam_unit;               /* repeat family unit length, 0 = none */
    uint32_t fam_copies;             /* copies per family */
    uint32_t fam_count;              /* number of families */
    double fam_div_min, fam_div_max;
    double n_frac;                   /* fraction of bases shown as N blocks */
    uint32_t n_block_min, n_block_max;
} gs_synth_ref_spec;

#define GS_LEN_FIXED 0
#define GS_LEN_CHOICE 1
#define GS_LEN_LOGNORMAL 2
#define GS_LEN_UNIFORM 3

typedef struct {
    uint64_t seed;
    uint32_t n_reads;
    uint32_t len_mode;
    uint32_t len_fixed;
    uint32_t n_choices;
    uint32_t len_choices[8];
    double ln_median, ln_sigma;
    uint32_t len_min, len_max;       /* clip (lognormal) or range (uniform) */
    double sub_rate;
    double indel_rate;               /* per base, half insertions, half deletions */
    uint32_t indel_max;              /* indel length 1..indel_max */
    double nrun_frac;                /* fraction of reads carrying an N run */
    uint32_t nrun_min, nrun_max;
} gs_synth_read_spec;

/* codes: length bytes of 0..3 (the indexed text: bases under N blocks are the
 * generated bases).  nmask: NULL or length bytes, 1 where the sequence shows N. */
int gs_synth_reference(const gs_synth_ref_spec *spec, uint8_t *codes, uint8_t *nmask,
                       int n_threads);
/* Upper bound of the bytes gs_synth_reads writes into seqs. */
uint64_t gs_synth_reads_capacity(const gs_synth_read_spec *spec);
/* ASCII reads (ACGTN) sampled from both strands; offsets/lengths per read. */
int gs_synth_reads(const uint8_t *codes, const uint8_t *nmask, uint64_t length,
                   const gs_synth_read_spec *spec, char *seqs, uint64_t seqs_cap,
                   uint64_t *offsets, uint32_t *lengths, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
