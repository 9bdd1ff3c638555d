/* abi_check.c — the C ABI (include/tuna_gpu.h) from plain C11: the header
 * compiles as C, the program links against libtuna_gpu.so, and every entry
 * point answers a null or out-of-range argument with its documented status
 * without touching a device. argv[1]: a file for tg_read_input. */
#include <stdio.h>
#include <string.h>

#include "tuna_gpu.h"

static int fails = 0;
#define EXPECT(cond)                                                  \
    do {                                                              \
        if (!(cond)) {                                                \
            ++fails;                                                  \
            printf("FAIL line %d: %s\n", __LINE__, #cond);            \
        }                                                             \
    } while (0)

static int sink(const void* data, size_t bytes, uint64_t pairs, void* user) {
    (void)data; (void)bytes; (void)pairs; (void)user;
    return 0;
}
static int part_sink(uint32_t part, const uint8_t* data, size_t len, void* user) {
    (void)part; (void)data; (void)len; (void)user;
    return 0;
}

int main(int argc, char** argv) {
    tg_ctx* ctx = NULL;
    tg_job* job = NULL;
    tg_job_opts jo;
    tg_stats st;
    uint64_t n = 0, offs[2];
    size_t len = 0;
    char err[128];
    memset(&jo, 0, sizeof jo);
    jo.k = 31;
    jo.m = 21;

    EXPECT(strstr(tg_version(), "tuna-gb300") != NULL);
    EXPECT(tg_device_count() >= 0);
    EXPECT(tg_ctx_create(NULL, NULL) == TG_ERR_ARG);
    if (tg_device_count() == 0) {
        EXPECT(tg_ctx_create(NULL, &ctx) == TG_ERR_CUDA && ctx == NULL);
    }
    EXPECT(tg_ctx_destroy(NULL) == TG_ERR_ARG);
    EXPECT(tg_last_error(NULL) != NULL);
    EXPECT(tg_ctx_stream(NULL) == NULL);

    EXPECT(tg_job_begin(NULL, &jo, &job) == TG_ERR_ARG);
    EXPECT(tg_job_feed_seq(NULL, (const uint8_t*)"ACGT", 4) == TG_ERR_ARG);
    EXPECT(tg_job_feed_seq_device(NULL, NULL, 0) == TG_ERR_ARG);
    EXPECT(tg_job_feed_fastx(NULL, (const uint8_t*)">a\nACGT\n", 8) == TG_ERR_ARG);
    EXPECT(tg_job_feed_fastx_device(NULL, NULL, 0) == TG_ERR_ARG);
    EXPECT(tg_job_feed_file(NULL, "x.fa") == TG_ERR_ARG);
    EXPECT(tg_job_next_sample(NULL) == TG_ERR_ARG);
    EXPECT(tg_job_set_shard(NULL, 0, 1) == TG_ERR_ARG);
    EXPECT(tg_job_run(NULL) == TG_ERR_ARG);
    EXPECT(tg_job_stats(NULL, &st) == TG_ERR_ARG);
    EXPECT(tg_job_result_size(NULL) == 0);
    EXPECT(tg_job_key_words(NULL) == 0);
    EXPECT(tg_job_sample_count(NULL) == 0);
    EXPECT(tg_job_sample_offsets(NULL, offs) == TG_ERR_ARG);
    EXPECT(tg_job_result_copy(NULL, NULL, NULL, 0, 0) == TG_ERR_ARG);
    EXPECT(tg_job_drain(NULL, TG_FMT_TSV, sink, NULL) == TG_ERR_ARG);
    EXPECT(tg_job_write(NULL, TG_FMT_KFF, "out.kff") == TG_ERR_ARG);
    EXPECT(tg_job_export_partitions(NULL, part_sink, NULL) == TG_ERR_ARG);
    EXPECT(tg_job_end(NULL) == TG_ERR_ARG);

    EXPECT(tg_count_seq(NULL, &jo, (const uint8_t*)"ACGT", 4, NULL, NULL, 0, &n, &st) == TG_ERR_ARG);
    EXPECT(tg_count_fastx(NULL, &jo, (const uint8_t*)">a\nACGT\n", 8, NULL, NULL, 0, &n, &st) == TG_ERR_ARG);
    EXPECT(tg_count_batch(NULL, &jo, 0, NULL, NULL, NULL, NULL, NULL, 0, &n, &st) == TG_ERR_ARG);
    EXPECT(tg_count_batch_fastx(NULL, &jo, 0, NULL, NULL, NULL, NULL, NULL, 0, &n, &st) == TG_ERR_ARG);
    EXPECT(tg_fastx_to_stream(NULL, NULL, 0, NULL, 0, &len) == TG_ERR_ARG);

    err[0] = 0;
    EXPECT(tg_count_seq_device_noalloc(NULL, NULL, 0, NULL, NULL, 0, &n, NULL, err, sizeof err) == TG_ERR_ARG);
    EXPECT(err[0] != 0);
    jo.k = 64;
    EXPECT(tg_count_seq_device_noalloc(&jo, NULL, 0, NULL, NULL, 0, &n, NULL, err, sizeof err) ==
           TG_ERR_UNSUPPORTED);
    jo.k = 31;
    EXPECT(tg_count_seq_device_noalloc(&jo, (const uint8_t*)"x", TG_NOALLOC_MAX_LEN + 1u, NULL, NULL, 0, &n, NULL,
                                       err, sizeof err) == TG_ERR_ARG);
    /* gpu_parts: 0 or a power of two up to 4096, checked before any device work */
    {
        const uint32_t bad_parts[] = {3u, 8192u, 0x80000000u, 0xFFFFFFFFu};
        for (size_t i = 0; i < sizeof bad_parts / sizeof bad_parts[0]; ++i) {
            jo.gpu_parts = bad_parts[i];
            err[0] = 0;
            EXPECT(tg_count_seq_device_noalloc(&jo, (const uint8_t*)"ACGT", 4, NULL, NULL, 0, &n, NULL, err,
                                               sizeof err) == TG_ERR_ARG);
            EXPECT(strstr(err, "gpu_parts") != NULL);
        }
        jo.gpu_parts = 0;
    }

    EXPECT(tg_job_set_spill(NULL, 0, NULL) == TG_ERR_ARG);
    EXPECT(tg_read_input(NULL, 1, NULL, 0, &len, err, sizeof err) == TG_ERR_ARG);
    if (argc > 1) {
        uint8_t buf[256];
        EXPECT(tg_read_input(argv[1], 2, buf, sizeof buf, &len, err, sizeof err) == TG_OK);
        EXPECT(len == 9 && memcmp(buf, ">a\nACGTA\n", 9) == 0);
        EXPECT(tg_read_input(argv[1], 2, buf, 4, &len, err, sizeof err) == TG_ERR_ARG && len == 9);
    }
    EXPECT(tg_read_input("/nonexistent/in.fa", 1, NULL, 0, &len, err, sizeof err) == TG_ERR_IO);

    if (fails) {
        printf("%d checks failed\n", fails);
        return 1;
    }
    printf("OK\n");
    return 0;
}
