/* pipeline_chunks.h -- the chunk schedule of the host-sample pipeline
 * (xs_lookup_samples with host arrays, xs_run_event with host outputs).
 *
 * A batch of n lookups is cut into chunks that rotate over the pipeline's
 * streams.  Whole chunks hold `chunk` lookups; at each end of a batch longer
 * than 2.75 chunks a ramp of chunk/8, chunk/4, chunk/2 keeps the first copy
 * in and the last copy out short, since no other chunk's lookups overlap
 * them (large problem, 2M-lookup chunks: the last chunk's macro_xs alone took
 * 0.43 ms of a 19 ms run to come back; with the ramp the run went from 888 to
 * 905 M lookups/s).  The middle is cut into equal chunks of whole tiles.
 *
 * Plain C (also compiled by the CPU tests); capi.cu includes it.
 */
#ifndef XSGB_PIPELINE_CHUNKS_H
#define XSGB_PIPELINE_CHUNKS_H

/* Lookups per whole chunk: 2^21 for the plain kernel, 2^22 for the batched
 * one (each chunk is sorted on its own, and its persistent launch ends in a
 * tail), doubled while two of them fit in an eighth of the batch, at most
 * 2^24; never below one tile. */
static inline long xsgb_pipeline_whole(long n, int batched, long tile)
{
    long whole = batched ? (1L << 22) : (1L << 21);
    while (whole < (1L << 24) && whole * 2 <= n / 8) whole *= 2;
    return whole > tile ? whole : tile;
}

/* The chunk sizes of a batch of n > 0 lookups (chunk >= tile > 0): returns
 * how many; writes them to sizes[0 .. max) when sizes is not NULL. */
static inline long xsgb_pipeline_chunks(long n, long chunk, long tile, long *sizes, long max)
{
    long count = 0;
#define XSGB_PUSH(v)                                  \
    do {                                              \
        if (sizes && count < max) sizes[count] = (v); \
        count++;                                      \
    } while (0)
    const long r0 = chunk / 8, r1 = chunk / 4, r2 = chunk / 2;
    const long ends = 2 * (r0 + r1 + r2);
    if (n <= ends + chunk || r0 < tile) {
        for (long c0 = 0; c0 < n; c0 += chunk) XSGB_PUSH(n - c0 < chunk ? n - c0 : chunk);
        return count;
    }
    XSGB_PUSH(r0);
    XSGB_PUSH(r1);
    XSGB_PUSH(r2);
    const long mid = n - ends;
    const long k = (mid + chunk - 1) / chunk;
    long each = ((mid + k - 1) / k + tile - 1) / tile * tile;   /* whole tiles */
    if (each > chunk) each = chunk;
    for (long left = mid; left > 0; left -= each) XSGB_PUSH(left < each ? left : each);
    XSGB_PUSH(r2);
    XSGB_PUSH(r1);
    XSGB_PUSH(r0);
#undef XSGB_PUSH
    return count;
}

#endif
