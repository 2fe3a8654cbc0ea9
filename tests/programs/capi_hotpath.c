/* A C99 caller of the C interface, compiled against include/compute_c.h and
 * linked with libgbcompute.so: the device, buffer and algorithm checks that
 * the reference's C interface test makes (lib/test/Compute/capi.c:52-157),
 * with the same recipe and known answers: N = 10007 elements
 * host[i] = (i * 7919) % 1000 - 500, whose int32 sum, maximum (499),
 * inclusive scan, half-scaling transform, positive count and ascending sort
 * are checked on the host; a fill past the buffer, a 64-bit key sort and a
 * malformed expression must be rejected with the reference's statuses. The
 * user-kernel checks of that file are left out: those entry points return
 * CLC_ERROR_UNSUPPORTED here by design. Exit status = failed checks. */
#include <compute_c.h>

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int failed = 0, total = 0;

static void expect(int ok, const char* what, int line)
{
    ++total;
    if (!ok) {
        ++failed;
        fprintf(stderr, "check failed at line %d: %s (last error: %s)\n", line, what, clc_last_error());
    }
}
#define EXPECT(c) expect((c) != 0, #c, __LINE__)
#define SUCCEEDS(call) expect((call) == CLC_SUCCESS, #call, __LINE__)

static void devices_and_buffers(clc_context ctx)
{
    size_t count = 0;
    clc_device_info info;
    int32_t data[64], back[64];
    clc_buffer a = NULL, b = NULL, none = NULL;
    int i;

    SUCCEEDS(clc_device_count(&count));
    EXPECT(count > 0);
    SUCCEEDS(clc_device_get_info(0, &info));
    EXPECT(strlen(info.name) > 0 && info.is_gpu == 1);
    EXPECT(clc_device_get_info(count, &info) == CLC_ERROR_INVALID_ARGUMENT);
    EXPECT(strlen(clc_last_error()) > 0);
    EXPECT(clc_device_count(NULL) == CLC_ERROR_INVALID_ARGUMENT);

    for (i = 0; i < 64; ++i) data[i] = 11 * i - 300;
    SUCCEEDS(clc_buffer_alloc(ctx, sizeof data, &a));
    SUCCEEDS(clc_buffer_alloc(ctx, sizeof data, &b));
    SUCCEEDS(clc_buffer_alloc(ctx, 0, &none));
    EXPECT(clc_buffer_size(a) == sizeof data && clc_buffer_size(none) == 0);
    SUCCEEDS(clc_buffer_write(ctx, a, 0, sizeof data, data));
    /* elements 8..47 of a land at the front of b */
    SUCCEEDS(clc_buffer_copy(ctx, a, 8 * sizeof(int32_t), b, 0, 40 * sizeof(int32_t)));
    memset(back, 0, sizeof back);
    SUCCEEDS(clc_buffer_read(ctx, b, 0, 40 * sizeof(int32_t), back));
    EXPECT(memcmp(back, data + 8, 40 * sizeof(int32_t)) == 0);
    EXPECT(clc_buffer_read(ctx, a, 8, sizeof data, back) == CLC_ERROR_INVALID_ARGUMENT);
    EXPECT(clc_buffer_write(ctx, none, 0, 0, NULL) == CLC_SUCCESS);
    clc_buffer_release(a);
    clc_buffer_release(b);
    clc_buffer_release(none);
    clc_buffer_release(NULL);
}

static void algorithms(clc_context ctx)
{
    enum { N = 10007 };
    int32_t* h = (int32_t*)malloc(N * sizeof(int32_t));
    int32_t* r = (int32_t*)malloc(N * sizeof(int32_t));
    float* f = (float*)malloc(N * sizeof(float));
    double* dh = (double*)malloc(N * sizeof(double));
    clc_buffer in = NULL, out = NULL, fb = NULL, db = NULL;
    int64_t sum64 = 0;
    int32_t run = 0, init = 0, got = 0, largest = 0, zero = 0, start = 5, step = 2;
    double dsum_host = 0.0, dsum = 0.0, dinit = 0.0;
    size_t positives = 0, kept = 0, i;
    int scan_ok = 1, sorted = 1;

    for (i = 0; i < N; ++i) {
        h[i] = (int32_t)((i * 7919u) % 1000u) - 500;
        sum64 += h[i];
        positives += h[i] > 0;
        dh[i] = 0.25 * (double)h[i];
        dsum_host += dh[i];
    }
    SUCCEEDS(clc_buffer_alloc(ctx, N * sizeof(int32_t), &in));
    SUCCEEDS(clc_buffer_alloc(ctx, N * sizeof(int32_t), &out));
    SUCCEEDS(clc_buffer_alloc(ctx, N * sizeof(float), &fb));
    SUCCEEDS(clc_buffer_write(ctx, in, 0, N * sizeof(int32_t), h));

    /* reduce: the int32 sum wraps like the int64 sum cast to int32 */
    SUCCEEDS(clc_reduce(ctx, in, N, CLC_TYPE_I32, "(a + b)", "0", &init, &got));
    EXPECT(got == (int32_t)sum64);
    init = INT32_MIN;
    SUCCEEDS(clc_reduce(ctx, in, N, CLC_TYPE_I32, "max(a, b)", "INT_MIN", &init, &largest));
    EXPECT(largest == 499);

    /* inclusive scan, every element checked */
    SUCCEEDS(clc_scan(ctx, in, out, N, CLC_TYPE_I32, "(a + b)", "0", 0));
    SUCCEEDS(clc_buffer_read(ctx, out, 0, N * sizeof(int32_t), r));
    for (i = 0; i < N; ++i) {
        run += h[i];
        if (r[i] != run) scan_ok = 0;
    }
    EXPECT(scan_ok && r[N - 1] == (int32_t)sum64);

    /* transform to float */
    SUCCEEDS(clc_transform(ctx, in, CLC_TYPE_I32, fb, CLC_TYPE_F32, N, "(float)x * 0.5f"));
    SUCCEEDS(clc_buffer_read(ctx, fb, 0, N * sizeof(float), f));
    EXPECT(f[3] == (float)h[3] * 0.5f && f[N - 1] == (float)h[N - 1] * 0.5f);

    /* copy_if keeps the positive elements */
    SUCCEEDS(clc_copy_if(ctx, in, out, N, CLC_TYPE_I32, "x > 0", &kept));
    EXPECT(kept == positives);

    /* sort in place, ascending */
    SUCCEEDS(clc_sort(ctx, in, CLC_TYPE_I32, NULL, N, 0));
    SUCCEEDS(clc_buffer_read(ctx, in, 0, N * sizeof(int32_t), r));
    for (i = 1; i < N; ++i)
        if (r[i - 1] > r[i]) sorted = 0;
    EXPECT(sorted);

    /* sequence and fill */
    SUCCEEDS(clc_sequence(ctx, out, N, CLC_TYPE_I32, &start, &step));
    SUCCEEDS(clc_buffer_read(ctx, out, 0, N * sizeof(int32_t), r));
    EXPECT(r[0] == 5 && r[N - 1] == 5 + 2 * (N - 1));
    SUCCEEDS(clc_fill(ctx, out, N, CLC_TYPE_I32, &zero));
    SUCCEEDS(clc_buffer_read(ctx, out, 0, N * sizeof(int32_t), r));
    EXPECT(r[0] == 0 && r[N - 1] == 0);

    /* the rejections the reference pins */
    EXPECT(clc_fill(ctx, out, N + 1, CLC_TYPE_I32, &zero) == CLC_ERROR_INVALID_ARGUMENT);
    EXPECT(clc_sort(ctx, out, CLC_TYPE_I64, NULL, N / 2, 0) == CLC_ERROR_INVALID_ARGUMENT);
    EXPECT(clc_transform(ctx, in, CLC_TYPE_I32, out, CLC_TYPE_I32, N, "x +* nonsense") == CLC_ERROR_BUILD);
    EXPECT(strstr(clc_last_error(), "build log") != NULL);

    /* double reduce (the device has fp64) */
    SUCCEEDS(clc_buffer_alloc(ctx, N * sizeof(double), &db));
    SUCCEEDS(clc_buffer_write(ctx, db, 0, N * sizeof(double), dh));
    SUCCEEDS(clc_reduce(ctx, db, N, CLC_TYPE_F64, "(a + b)", "0.0", &dinit, &dsum));
    EXPECT(fabs(dsum - dsum_host) <= 1e-9 * fabs(dsum_host) + 1e-9);

    SUCCEEDS(clc_finish(ctx));
    clc_buffer_release(in);
    clc_buffer_release(out);
    clc_buffer_release(fb);
    clc_buffer_release(db);
    free(h);
    free(r);
    free(f);
    free(dh);
}

int main(void)
{
    clc_context ctx = NULL;
    if (clc_context_create(CLC_DEFAULT_DEVICE, &ctx) != CLC_SUCCESS) {
        fprintf(stderr, "no context: %s\n", clc_last_error());
        return 1;
    }
    devices_and_buffers(ctx);
    algorithms(ctx);
    clc_context_release(ctx);
    printf("%d of %d checks failed\n", failed, total);
    return failed;
}
