/*
 * Harness around the reference's own CPU join, JoinProvider::join_cpu
 * (src/join/join_provider.cuh:241-284), compiled from the reference sources by
 * oracle/ref_build.sh. Test infrastructure only.
 *
 * JoinProvider::join dispatches host tables to join_cpu (cuh:230-233). With
 * JoinConfig::devices = 0 the constructor's device loop (cuh:517-564) makes no CUDA call,
 * so this runs on a machine without a GPU.
 *
 * usage: ref_join_cpu <in.bin> <out.bin>
 *   in:  u64 column_count, u64 |R|, u64 |S|, then R column_values (|R|*cc u64),
 *        R primary_keys (|R| u64), S column_values, S primary_keys
 *   out: u64 |RS|, then the rs table's column_values ([r_pk, s_pk] per row)
 */
#include <algorithm>
#include <cstring>
#include <memory>
#include "join/join_provider.cuh"
#include <cstdio>
#include <vector>

static bool read_u64(FILE *f, unsigned long long *dst, size_t n) {
    return fread(dst, sizeof(unsigned long long), n, f) == n;
}

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s in out\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    unsigned long long hdr[3];
    if (!f || !read_u64(f, hdr, 3)) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 3;
    }
    size_t cc = hdr[0];
    db_table r(cc, hdr[1], false);
    db_table s(cc, hdr[2], false);
    bool ok = read_u64(f, r.column_values, r.size * cc) && read_u64(f, r.primary_keys, r.size) && read_u64(f, s.column_values, s.size * cc) && read_u64(f, s.primary_keys, s.size);
    fclose(f);
    if (!ok) {
        fprintf(stderr, "short input\n");
        return 3;
    }
    JoinConfig config;
    config.devices = 0;
    config.profile_enabled = false;
    db_table rs;
    JoinStatus status;
    {
        JoinProvider provider(config);
        status = provider.join(r, s, rs);
    }
    if (!status.successful) {
        fprintf(stderr, "join failed: %s\n", status.message.c_str());
        return 4;
    }
    f = fopen(argv[2], "wb");
    unsigned long long m = rs.size;
    fwrite(&m, sizeof(m), 1, f);
    if (m) {
        fwrite(rs.column_values, sizeof(unsigned long long), 2 * m, f);
    }
    fclose(f);
    rs.free();
    r.free();
    s.free();
    return 0;
}
