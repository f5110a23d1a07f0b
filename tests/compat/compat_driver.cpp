// Drives the reference API names (include/vj_compat.hpp) the way the reference's drivers
// do -- src/playground/probe_benchmark.cu:106-152 (hash_func + build_and_probe_gpu),
// src/join/join_provider.cuh:586-595 (set_radix_width + partition_gpu) and
// src/join_benchmark.cu:246-265 (JoinProvider::join on device and on host tables) -- and
// writes every result to a binary file that tests/test_compat_gpu.py checks against the
// CPU oracle.
//
// usage: compat_driver <in.bin> <out.bin>
//   in:  u64 column_count, u64 |R|, u64 |S|, R column_values, R primary_keys,
//        S column_values, S primary_keys   (db_table layout)
//   out: u64 records, each: u64 tag, u64 length, length u64 values
//        tag 1: hashes of R (hash_func, HASH_BITS/HASH_CHUNK_BITS of this build)
//        tag 2: partition histogram of R, tag 3: partition offsets of R
//        tag 4: partitioned R primary keys, tag 5: partitioned R hashes
//        tag 6: build_and_probe_gpu pairs, tag 7: JoinProvider::join (device) pairs
//        tag 8: JoinProvider::join (host tables) pairs, tag 9: status flags
#include "vj_compat.hpp"

#include <cstdio>
#include <vector>

static std::vector<unsigned long long> records;

static void emit(unsigned long long tag, const std::vector<unsigned long long> &v) {
    records.push_back(tag);
    records.push_back(v.size());
    records.insert(records.end(), v.begin(), v.end());
}

template <typename T>
static std::vector<unsigned long long> from_device(const T *d, size_t n) {
    std::vector<T> h(n);
    if (n) cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
    return std::vector<unsigned long long>(h.begin(), h.end());
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *f = fopen(argv[1], "rb");
    unsigned long long hdr[3];
    if (!f || fread(hdr, 8, 3, f) != 3) return 3;
    const size_t cc = hdr[0];
    db_table h_r(cc, hdr[1], false), h_s(cc, hdr[2], false);
    bool ok = fread(h_r.column_values, 8, h_r.size * cc, f) == h_r.size * cc && fread(h_r.primary_keys, 8, h_r.size, f) == h_r.size && fread(h_s.column_values, 8, h_s.size * cc, f) == h_s.size * cc &&
              fread(h_s.primary_keys, 8, h_s.size, f) == h_s.size;
    fclose(f);
    if (!ok) return 3;
    std::vector<unsigned long long> flags;

    db_table r = h_r.copy(true), s = h_s.copy(true);
    cudaStream_t stream;
    cudaStreamCreate(&stream);

    // hash_func over the key columns, as JoinProvider::hash_table does (cuh:926-931)
    HashConfig hash_config;
    hash_config.algorithm = "fnv";
    hash_config.stream = stream;
    db_hash_table r_hash(r.size, true), s_hash(s.size, true);
    const short element_chunks = (short)(cc * sizeof(column_t) / sizeof(chunk_t));
    hash_func(r.size, 0, element_chunks, (chunk_t *)r.column_values, r_hash.hashes, hash_config);
    flags.push_back(hash_config.last_status);
    hash_func(s.size, 0, element_chunks, (chunk_t *)s.column_values, s_hash.hashes, hash_config);
    cudaStreamSynchronize(stream);
    emit(1, from_device(r_hash.hashes, r.size));

    // an unknown algorithm launches nothing and reports it (the reference is silent)
    HashConfig bad;
    bad.algorithm = "xor_hw";
    hash_func(r.size, 0, element_chunks, (chunk_t *)r.column_values, r_hash.hashes, bad);
    flags.push_back(bad.last_status);

    // one radix pass of R on bits [4, 10) of the hash
    PartitionConfig part;
    part.stream = stream;
    part.set_radix_width(6);
    db_table r_swap(cc, r.size, true);
    db_hash_table r_hash_swap(r.size, true);
    std::vector<index_t> hist(part.bins), offs(part.bins);
    partition_gpu(r, r_hash, r_swap, r_hash_swap, 4, hist.data(), offs.data(), part);
    flags.push_back(part.last_status);
    emit(2, std::vector<unsigned long long>(hist.begin(), hist.end()));
    emit(3, std::vector<unsigned long long>(offs.begin(), offs.end()));
    emit(4, from_device(r_swap.primary_keys, r.size));
    emit(5, from_device(r_hash_swap.hashes, r.size));

    // build_and_probe_gpu on the unpartitioned tables (probe_benchmark.cu:143)
    ProbeConfig probe;
    probe.probe_mode = ProbeConfig::MODE_GLOBAL_R;
    probe.build_table_load = 0.25f;
    probe.stream = stream;
    db_table rs;
    JoinStatus st = build_and_probe_gpu(r, r_hash, s, s_hash, rs, 0, probe);
    flags.push_back(st.successful ? 0 : 1);
    emit(6, from_device(rs.column_values, 2 * rs.size));
    rs.free();

    // JoinProvider::join on device tables and on host tables (join_benchmark.cu:246, :253)
    JoinConfig jc;
    jc.buckets = 256;
    jc.hash_config.algorithm = "fnv";
    jc.probe_config = probe;
    JoinProvider provider(jc);
    db_table rs_dev;
    st = provider.join(r, s, rs_dev);
    flags.push_back(st.successful ? 0 : 1);
    flags.push_back(provider.get_join_summary().rs_elements);
    emit(7, from_device(rs_dev.column_values, 2 * rs_dev.size));
    db_table rs_host;
    st = provider.join(h_r, h_s, rs_host);
    flags.push_back(st.successful ? 0 : 1);
    emit(8, std::vector<unsigned long long>(rs_host.column_values, rs_host.column_values + 2 * rs_host.size));
    emit(9, flags);

    rs_dev.free();
    rs_host.free();
    r_swap.free();
    r_hash_swap.free();
    r_hash.free();
    s_hash.free();
    r.free();
    s.free();
    part.free();
    cudaStreamDestroy(stream);

    f = fopen(argv[2], "wb");
    unsigned long long nrec = records.size();
    fwrite(&nrec, 8, 1, f);
    fwrite(records.data(), 8, records.size(), f);
    fclose(f);
    return 0;
}
