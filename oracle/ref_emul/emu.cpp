/*
 * emu.cpp -- runs the reference's own kernel bodies on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  build_ref.py cuts the kernels out of the
 * reference's seed_gen.cu into _ref/ref_kernels.inc; this file supplies
 *   - a launch emulator: blocks and threads of a grid run one after another,
 *     each seeing its own threadIdx/blockIdx;
 *   - a warp emulator for find_seed_intervals_gpu: the 32 threads of a warp
 *     run as coroutines and every __shfl_up_sync is a rendezvous of all
 *     threads of the warp that have not exited (the independent-thread-
 *     scheduling rule of sm_70 and later); a thread reading a lane that has
 *     exited gets that lane's last published value;
 *   - host versions of the CUB device calls main() makes (select, scan,
 *     reduce, stable segmented radix sort on the low bits);
 *   - ref_run(): the body of main()'s batch loop (seed_gen.cu:2917-3647),
 *     with device buffers as zeroed host buffers and the <<<1,1>>> wrappers
 *     (seed_gen.cu:687-724, :1224-1251) inlined, writing the text records.
 */
#include "shim.h"

#include <ucontext.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <string>
#include <thread>
#include <vector>

thread_local EmuThread *emu_cur;

#include "ref_kernels.inc"

/* ------------------------------------------------------------------ */
/* launches */

static void launch(uint64_t grid, unsigned block, const std::function<void()> &body)
{
    EmuThread t;
    t.bdim = {block, 1, 1};
    for (uint64_t b = 0; b < grid; b++)
        for (unsigned x = 0; x < block; x++) {
            t.bid = {(unsigned)b, 0, 0};
            t.tid = {x, 0, 0};
            emu_cur = &t;
            body();
        }
}

static void launch_parallel(uint64_t grid, unsigned block, const std::function<void()> &body)
{
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint64_t> next(0);
    std::vector<std::thread> th;
    for (unsigned i = 0; i < nt; i++)
        th.emplace_back([&]() {
            EmuThread t;
            t.bdim = {block, 1, 1};
            for (;;) {
                uint64_t b = next.fetch_add(64);
                if (b >= grid) break;
                for (uint64_t bb = b; bb < b + 64 && bb < grid; bb++)
                    for (unsigned x = 0; x < block; x++) {
                        t.bid = {(unsigned)bb, 0, 0};
                        t.tid = {x, 0, 0};
                        emu_cur = &t;
                        body();
                    }
            }
        });
    for (auto &x : th) x.join();
}

/* warp emulator */
enum { L_RUN, L_WAIT, L_EXIT };
struct Lane {
    EmuThread t;
    ucontext_t uc;
    int state;
    uint32_t val, result;
    unsigned delta;
    std::vector<char> stack;
};
struct Warp {
    Lane lane[32];
    ucontext_t sched;
    int cur;
    const std::function<void()> *body;
};
static thread_local Warp *g_warp;

static void lane_main(int i)
{
    Warp *w = g_warp;
    emu_cur = &w->lane[i].t;
    (*w->body)();
    w->lane[i].state = L_EXIT;
    /* uc_link returns to the scheduler */
}

uint32_t emu_shfl_up(uint32_t mask, uint32_t v, unsigned delta)
{
    (void)mask;
    Warp *w = g_warp;
    if (!w) return v;
    Lane &L = w->lane[w->cur];
    L.val = v;
    L.delta = delta;
    L.state = L_WAIT;
    swapcontext(&L.uc, &w->sched);
    emu_cur = &L.t;
    return L.result;
}

static void launch_warps(uint64_t grid, unsigned block, const std::function<void()> &body)
{
    Warp *w = new Warp();
    w->body = &body;
    for (auto &L : w->lane) L.stack.resize(1 << 18);
    g_warp = w;
    for (uint64_t b = 0; b < grid; b++) {
        for (unsigned w0 = 0; w0 < block; w0 += 32) {
            for (int i = 0; i < 32; i++) {
                Lane &L = w->lane[i];
                L.t.bdim = {block, 1, 1};
                L.t.bid = {(unsigned)b, 0, 0};
                L.t.tid = {w0 + (unsigned)i, 0, 0};
                L.state = L_RUN;
                L.val = 0;
                getcontext(&L.uc);
                L.uc.uc_stack.ss_sp = L.stack.data();
                L.uc.uc_stack.ss_size = L.stack.size();
                L.uc.uc_link = &w->sched;
                makecontext(&L.uc, (void (*)())lane_main, 1, i);
            }
            for (;;) {
                for (int i = 0; i < 32; i++)
                    if (w->lane[i].state == L_RUN) {
                        w->cur = i;
                        swapcontext(&w->sched, &w->lane[i].uc);
                    }
                int waiting = 0;
                for (int i = 0; i < 32; i++) waiting += w->lane[i].state == L_WAIT;
                if (!waiting) break;
                for (int i = 0; i < 32; i++) {
                    Lane &L = w->lane[i];
                    if (L.state != L_WAIT) continue;
                    int src = i - (int)L.delta;
                    L.result = src >= 0 ? w->lane[src].val : L.val;
                }
                for (int i = 0; i < 32; i++)
                    if (w->lane[i].state == L_WAIT) w->lane[i].state = L_RUN;
            }
        }
    }
    g_warp = NULL;
    delete w;
}

/* ------------------------------------------------------------------ */
/* host versions of the CUB calls */

static uint32_t select_flagged(const uint32_t *in, const uint16_t *flags, uint32_t *out, uint64_t n)
{
    uint32_t k = 0;
    for (uint64_t i = 0; i < n; i++)
        if (flags[i]) out[k++] = in[i];
    return k;
}

static void exclusive_sum(const uint32_t *in, uint32_t *out, uint64_t n)
{
    uint32_t s = 0;
    for (uint64_t i = 0; i < n; i++) {
        uint32_t v = in[i];
        out[i] = s;
        s += v;
    }
}

template <class V>
static void seg_sort(const uint64_t *kin, uint64_t *kout, const V *vin, V *vout, uint64_t n_items,
                     int n_seg, const uint32_t *beg, const uint32_t *end, int bits)
{
    (void)n_items;
    uint64_t mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
    std::vector<uint64_t> idx;
    for (int s = 0; s < n_seg; s++) {
        uint32_t b = beg[s], e = end[s];
        idx.clear();
        for (uint32_t i = b; i < e; i++) idx.push_back(i);
        std::stable_sort(idx.begin(), idx.end(),
                         [&](uint64_t x, uint64_t y) { return (kin[x] & mask) < (kin[y] & mask); });
        for (uint32_t i = b; i < e; i++) {
            kout[i] = kin[idx[i - b]];
            vout[i] = vin[idx[i - b]];
        }
    }
}

/* ------------------------------------------------------------------ */

#define BASE_BATCH_SIZE 1000000
#define OUTPUT_SIZE_MUL 3

/* n_fwd_out (may be NULL): per read, the forward records the reference's
 * search kept after its own pruning (n_smems_fow), the count its MEM filter
 * branches on (seed_gen.cu:1110-1113) */
extern "C" int ref_run(const char *prefix, const char *seqs, const uint64_t *offs,
                       const uint32_t *lens, uint32_t n_reads, int min_seed_size, int is_smem,
                       const char *out_path, uint32_t *n_fwd_out)
{
    bwt_t bwt;
    int pre_calc_seed_len = 13;
    size_t pl = strlen(prefix);
    char *fn = (char *)calloc(pl + 10, 1);
    strcpy(fn, prefix); strcat(fn, ".bwt"); bwt_restore_bwt(fn, &bwt);
    strcpy(fn, prefix); strcat(fn, ".sa"); bwt_restore_sa(fn, &bwt);
    free(fn);
    memset(L2_gpu, 0, sizeof(L2_gpu));
    memcpy(L2_gpu, bwt.L2, 5 * sizeof(bwtint_t));
    /* the uint4 loads of the last block may read past the .bwt words */
    bwt.bwt = (uint32_t *)realloc(bwt.bwt, (bwt.bwt_size + 16) * 4);
    memset(bwt.bwt + bwt.bwt_size, 0, 64);

    /* the 13-mer table of the last index is kept: tests call ref_run many
     * times on one index */
    static std::string cached_prefix;
    static std::vector<uint2> cached_table;
    uint64_t n_pat = 1ull << (pre_calc_seed_len << 1);
    std::string key = std::string(prefix) + ":" + std::to_string(bwt.primary) + ":" +
                      std::to_string(bwt.seq_len) + ":" + std::to_string(bwt.bwt_size);
    if (cached_prefix != key) {
        cached_table.assign(n_pat, uint2{0, 0});
        uint2 *t = cached_table.data();
        launch_parallel((n_pat + 127) / 128, 128, [&]() {
            pre_calc_seed_intervals_gpu(t, pre_calc_seed_len, bwt, (int)n_pat);
        });
        cached_prefix = key;
    }
    uint2 *pre_calc = cached_table.data();

    FILE *out = fopen(out_path, "w");
    if (!out) return -2;
    char *read_batch = (char *)malloc(BASE_BATCH_SIZE + 1000000 + 16);
    uint32_t *read_offsets = (uint32_t *)calloc(1000000, sizeof(uint32_t));
    uint32_t *read_sizes = (uint32_t *)calloc(1000000, sizeof(uint32_t));
    int reads_processed = 0, max_read_size = 0;
    uint32_t next = 0;
    int all_done = n_reads == 0;
    int status = 0;
    while (!all_done) {
        int total_reads = 0, read_batch_size = 0, prev_len = 0;
        while (read_batch_size < BASE_BATCH_SIZE) {
            if (next >= n_reads) { all_done = 1; break; }
            int L = (int)lens[next];
            memcpy(read_batch + read_batch_size, seqs + offs[next], L);
            read_batch_size += L;
            read_offsets[total_reads] = total_reads == 0 ? 0 : read_offsets[total_reads - 1] + prev_len;
            read_sizes[total_reads] = L;
            prev_len = L;
            total_reads++;
            if (L > max_read_size) max_read_size = L;
            next++;
        }
        if (total_reads == 0) break;
        int n_bits_max_read_size = (int)ceil(log2((double)max_read_size));
        int rbs8 = read_batch_size % 8 ? read_batch_size + (8 - read_batch_size % 8) : read_batch_size;
        int N2 = rbs8 - (min_seed_size - 1) * total_reads;

        uint8_t *read_batch_gpu = (uint8_t *)calloc(rbs8 + 16, 1);
        uint32_t *read_sizes_gpu = (uint32_t *)calloc(total_reads + 1, 4);
        uint32_t *read_offsets_gpu = (uint32_t *)calloc(total_reads + 1, 4);
        uint32_t *n_smems_fow = (uint32_t *)calloc(total_reads + 1, 4);
        uint32_t *n_smems_rev = (uint32_t *)calloc(total_reads + 1, 4);
        uint32_t *n_smems_fow_rev = read_sizes_gpu;
        uint32_t *n_smems_fow_rev_scan = (uint32_t *)calloc(total_reads + 2, 4);
        uint32_t *packed_fow = (uint32_t *)calloc((rbs8 >> 3) + 1, 4);
        uint32_t *packed_rev = (uint32_t *)calloc((rbs8 >> 3) + 1, 4);
        uint32_t *n_seeds_fow_rev_scan = (uint32_t *)calloc(2 * (uint64_t)N2 + 2, 4);
        uint32_t *thread_read_num = n_seeds_fow_rev_scan;
        uint32_t *thread_read_idx = &n_seeds_fow_rev_scan[N2];
        uint32_t *n_smems_sum_gpu = &n_smems_fow_rev_scan[total_reads];
        uint32_t n_seeds_sum_gpu = 0;
        uint32_t n_smems_max_gpu[2] = {0, 0};
        uint64_t big = (uint64_t)OUTPUT_SIZE_MUL * 2 * 2 * N2;
        uint2 *sip = (uint2 *)calloc(big + 1, sizeof(uint2));
        int2 *seed_read_pos = (int2 *)sip;
        uint2 *seed_intervals = &sip[2 * N2];
        uint2 *sipc = (uint2 *)calloc(big + 1, sizeof(uint2));
        int2 *seed_read_pos_compact = (int2 *)sipc;
        uint2 *seed_intervals_compact = &sipc[2 * N2];
        uint32_t *nsf = (uint32_t *)calloc(big + 1, 4);
        uint32_t *n_seeds_fow_rev = nsf;
        uint32_t *is_smem_flag = &nsf[2 * N2];
        uint32_t *seed_ref_pos_gpu = is_smem ? NULL : (uint32_t *)calloc(big + 1, 4);
        uint32_t *n_ref_pos = read_offsets_gpu;

        memcpy(read_batch_gpu, read_batch, read_batch_size);
        memcpy(read_offsets_gpu, read_offsets, total_reads * 4);
        memcpy(read_sizes_gpu, read_sizes, total_reads * 4);
        int BLOCKDIM = 128;
        int N_BLOCKS = ((rbs8 >> 3) + BLOCKDIM - 1) / BLOCKDIM;
        launch(N_BLOCKS, BLOCKDIM, [&]() { pack_4bit_rev((uint32_t *)read_batch_gpu, packed_rev, rbs8 >> 3); });
        launch(N_BLOCKS, BLOCKDIM, [&]() { pack_4bit_fow((uint32_t *)read_batch_gpu, packed_fow, rbs8 >> 3); });
        N_BLOCKS = ((total_reads * max_read_size) + BLOCKDIM - 1) / BLOCKDIM;
        launch(N_BLOCKS, BLOCKDIM, [&]() {
            prepare_batch(thread_read_num, thread_read_idx, read_offsets_gpu, read_sizes_gpu,
                          min_seed_size, total_reads * max_read_size, 0, max_read_size);
        });
        int n_seed_cands = read_batch_size - (total_reads * (min_seed_size - 1));
        memset(is_smem_flag, 0, 2 * (uint64_t)N2 * 4);
        memset(n_smems_fow, 0, total_reads * 4);
        memset(n_smems_rev, 0, total_reads * 4);
        N_BLOCKS = ((2 * n_seed_cands) + BLOCKDIM - 1) / BLOCKDIM;
        launch_warps(N_BLOCKS, BLOCKDIM, [&]() {
            find_seed_intervals_gpu(packed_fow, packed_rev, read_sizes_gpu, read_offsets_gpu,
                                    seed_intervals, seed_read_pos, thread_read_num, thread_read_idx,
                                    is_smem_flag, pre_calc, n_smems_fow, n_smems_rev, min_seed_size,
                                    bwt, pre_calc_seed_len, n_seed_cands);
        });
        for (int r = 0; r < total_reads; r++) {
            if (n_fwd_out) n_fwd_out[reads_processed + r] = n_smems_fow[r];
            n_smems_max_gpu[0] = std::max(n_smems_max_gpu[0], n_smems_fow[r]);
            n_smems_max_gpu[1] = std::max(n_smems_max_gpu[1], n_smems_rev[r]);
        }
        *n_smems_sum_gpu = select_flagged((uint32_t *)seed_intervals, (uint16_t *)is_smem_flag,
                                          (uint32_t *)seed_intervals_compact, 4 * (uint64_t)N2);
        *n_smems_sum_gpu = select_flagged((uint32_t *)seed_read_pos, (uint16_t *)is_smem_flag,
                                          (uint32_t *)seed_read_pos_compact, 4 * (uint64_t)N2);
        N_BLOCKS = (total_reads + BLOCKDIM - 1) / BLOCKDIM;
        launch(N_BLOCKS, BLOCKDIM, [&]() { sum_arrays(n_smems_fow, n_smems_rev, n_smems_fow_rev, total_reads); });
        exclusive_sum(n_smems_fow_rev, n_smems_fow_rev_scan, total_reads);
        memset(n_ref_pos, 0, total_reads * 4);
        uint32_t max_val = std::max(n_smems_max_gpu[0], n_smems_max_gpu[1]);
        int n_tasks = (int)(max_val * (uint32_t)total_reads);
        *n_smems_sum_gpu = *n_smems_sum_gpu / 2;
        int FB = (2 * n_tasks + 127) / 128;
        if (is_smem) {
            launch(FB, 128, [&]() {
                filter_seed_intervals_gpu(seed_intervals_compact, seed_read_pos_compact, n_smems_fow,
                                          n_smems_rev, n_smems_fow_rev_scan, max_val, n_tasks);
            });
            seg_sort<uint64_t>((uint64_t *)seed_read_pos_compact, (uint64_t *)seed_read_pos,
                               (uint64_t *)seed_intervals_compact, (uint64_t *)seed_intervals,
                               *n_smems_sum_gpu, total_reads, n_smems_fow_rev_scan,
                               n_smems_fow_rev_scan + 1, n_bits_max_read_size);
            launch(FB, 128, [&]() {
                count_seed_intervals_gpu(seed_intervals, n_smems_fow_rev, n_seeds_fow_rev,
                                         n_smems_fow_rev_scan, n_ref_pos, max_val << 1, 2 * n_tasks);
            });
        } else {
            launch(FB, 128, [&]() {
                filter_seed_intervals_gpu_mem(seed_intervals_compact, seed_read_pos_compact, seed_intervals,
                                              n_smems_fow, n_smems_rev, n_smems_fow_rev_scan, max_val,
                                              n_tasks);
            });
            launch(FB, 128, [&]() {
                count_seed_intervals_gpu_mem(seed_intervals, seed_read_pos_compact, n_smems_fow, n_smems_rev,
                                             n_seeds_fow_rev, n_smems_fow_rev_scan, n_ref_pos, max_val,
                                             n_tasks);
            });
            int2 *swap = seed_read_pos_compact;
            seed_read_pos_compact = seed_read_pos;
            seed_read_pos = swap;
        }
        uint32_t n_smems_sum = *n_smems_sum_gpu;
        n_seeds_sum_gpu = 0;
        for (uint32_t i = 0; i < n_smems_sum; i++) n_seeds_sum_gpu += n_seeds_fow_rev[i];
        exclusive_sum(n_seeds_fow_rev, n_seeds_fow_rev_scan, n_smems_sum);
        uint32_t *seed_sa_idx = n_seeds_fow_rev;
        uint32_t n_seeds_sum = n_seeds_sum_gpu;
        if ((uint64_t)n_seeds_sum > big) {
            status = -7;   /* the reference exits here (seed_gen.cu:3555-3558) */
            break;
        }
        int2 *final_pos;
        uint32_t *ref_pos;
        int LB = (int)((n_smems_sum * THREADS_PER_SMEM + 127) / 128);
        n_seeds_fow_rev_scan[n_smems_sum] = n_seeds_sum;
        if (is_smem) {
            launch(LB, 128, [&]() {
                seeds_to_threads(seed_read_pos_compact, seed_sa_idx, n_seeds_fow_rev_scan, seed_intervals,
                                 seed_read_pos, n_smems_sum);
            });
            launch((n_seeds_sum + 127) / 128, 128, [&]() { locate_seeds_gpu(seed_sa_idx, bwt, n_seeds_sum); });
            final_pos = seed_read_pos_compact;
            ref_pos = seed_sa_idx;
        } else {
            launch(LB, 128, [&]() {
                seeds_to_threads_mem(seed_read_pos_compact, seed_sa_idx, n_seeds_fow_rev_scan, seed_intervals,
                                     seed_read_pos, n_smems_sum);
            });
            launch((n_seeds_sum + 127) / 128, 128, [&]() { locate_seeds_gpu(seed_sa_idx, bwt, n_seeds_sum); });
            uint32_t *n_ref_pos_scan = n_smems_fow_rev_scan;
            *n_smems_sum_gpu = n_seeds_sum;
            exclusive_sum(n_ref_pos, n_ref_pos_scan, total_reads);
            seg_sort<uint32_t>((uint64_t *)seed_read_pos_compact, (uint64_t *)seed_read_pos, seed_sa_idx,
                               seed_ref_pos_gpu, n_seeds_sum, total_reads, n_ref_pos_scan,
                               n_ref_pos_scan + 1, n_bits_max_read_size);
            final_pos = seed_read_pos;
            ref_pos = seed_ref_pos_gpu;
        }
        /* records (seed_gen.cu:3625-3647) */
        char sign[2] = {'+', '-'};
        uint32_t j = 0;
        for (int i = 0; i < total_reads; i++) {
            fprintf(out, "/*===================================%s seeds in read no. %d (Read[begin, End] -> "
                         "starting position(s) on the reference)===================================*/\n",
                    is_smem ? "SMEM" : "MEM", reads_processed + i + 1);
            int prev_b = -1, prev_e = -1;
            for (uint32_t y = 0; y < n_ref_pos[i] && j < n_seeds_sum; j++, y++) {
                if (prev_b == final_pos[j].x && prev_e == final_pos[j].y)
                    fprintf(out, ", %c%u", sign[((uint32_t)final_pos[j].y) >> 31], ref_pos[j]);
                else
                    fprintf(out, "\nRead[%d, %d] -> %c%u", final_pos[j].x << 1 >> 1, final_pos[j].y << 1 >> 1,
                            sign[((uint32_t)final_pos[j].y) >> 31], ref_pos[j]);
                prev_b = final_pos[j].x;
                prev_e = final_pos[j].y;
            }
            fprintf(out, "\n");
        }
        reads_processed += total_reads;
        free(read_batch_gpu); free(read_sizes_gpu); free(read_offsets_gpu); free(n_smems_fow);
        free(n_smems_rev); free(n_smems_fow_rev_scan); free(packed_fow); free(packed_rev);
        free(n_seeds_fow_rev_scan); free(sip); free(sipc); free(nsf); free(seed_ref_pos_gpu);
    }
    fclose(out);
    free(read_batch); free(read_offsets); free(read_sizes);
    free(bwt.bwt); free(bwt.sa); free(bwt.L2);
    return status;
}
