// vj_compat.hpp -- the reference's C++ names and signatures over the vj C ABI.
//
// A translation unit that included the reference's "hash/hash.cu" and
// "join/join_provider.cuh" can include this header instead and link libvj.so:
//
//   reference (vgerber/vectorized-join)                 here
//   db_hash_table, db_table   src/base/types.hpp:25-266  same fields and methods
//   HashConfig, hash_func     src/hash/hash.cu:22-42, :507-557      -> vj_hash
//   PartitionConfig, partition_gpu
//                             src/join/join_provider.cu:95-175, :610-661 -> vj_partition
//   ProbeConfig, build_and_probe_gpu
//                             src/join/join_provider.cu:177-287, :669-847 -> vj_build_probe
//   JoinConfig, JoinProvider, JoinSummary
//                             src/join/join_provider.cuh:54-122, :222-429 -> vj_join
//
// Differences a caller can observe (all deliberate):
//   - CUDA and library errors come back as a failed JoinStatus (or HashConfig::last_status)
//     instead of exit() (src/base/debug.cuh:64-82);
//   - JoinProvider::join does not partition its inputs in place
//     (src/join/join_provider.cuh:659-663 reuses them as swap space);
//   - JoinProvider::join on host tables runs the GPU join on copies of them (the reference
//     runs its nested-loop join_cpu, src/join/join_provider.cuh:241-284); the result is the
//     same multiset of pairs;
//   - the multi-GPU modes (JoinConfig::devices > 1) run on device 0;
//   - an unknown hash algorithm name launches nothing, as in the reference, and sets
//     HashConfig::last_status to VJ_ERR_INVALID_ARGUMENT;
//   - the rs table's primary_keys are 1..M (the reference's GPU path leaves them unset).
//
// HASH_BITS (32/64) and HASH_CHUNK_BITS (8/32/64/128) keep their meaning: define them before
// including this header (defaults 64/64, as src/base/config.h:27-31).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "vj.h"

#ifndef HASH_BITS
#define HASH_BITS 64
#endif
#ifndef HASH_CHUNK_BITS
#define HASH_CHUNK_BITS 64
#endif

typedef unsigned long long index_t;
typedef unsigned int index_s_t;
typedef unsigned long long column_t;

#if HASH_BITS == 32
typedef unsigned int hash_t;
#elif HASH_BITS == 64
typedef unsigned long long hash_t;
#endif

#if HASH_CHUNK_BITS == 8
typedef char chunk_t;
#elif HASH_CHUNK_BITS == 32
typedef uint1 chunk_t;
#elif HASH_CHUNK_BITS == 64
typedef uint2 chunk_t;
#elif HASH_CHUNK_BITS == 128
typedef uint4 chunk_t;
#endif

namespace vj_compat {

// One library context per device, created on first use and kept for the process.
inline vj_ctx *context(int device = -1) {
    static std::mutex mu;
    static std::map<int, vj_ctx *> ctxs;
    if (device < 0) {
        cudaGetDevice(&device);
    }
    std::lock_guard<std::mutex> lock(mu);
    auto it = ctxs.find(device);
    if (it != ctxs.end()) {
        return it->second;
    }
    vj_ctx *c = nullptr;
    if (vj_ctx_create(device, 0, &c) != VJ_OK) {
        return nullptr;
    }
    ctxs[device] = c;
    return c;
}

inline std::string last_error() {
    char buf[512];
    vj_last_error(buf, sizeof(buf));
    return std::string(buf);
}

}  // namespace vj_compat

struct JoinStatus {
    std::string message = "Unknown";
    bool successful = false;

    JoinStatus(bool successful, std::string message) {
        this->successful = successful;
        this->message = message;
    }
    JoinStatus(bool successful) {
        this->successful = successful;
        this->message = successful ? "Successful" : "Failed";
    }
    JoinStatus() : JoinStatus(false, "Unknown") {}
    bool is_successful() { return successful; }
    bool has_failed() { return !successful; }
};

inline JoinStatus status_from(int st, const char *what) {
    if (st == VJ_OK) {
        return JoinStatus(true);
    }
    return JoinStatus(false, std::string(what) + ": " + vj_status_string(st) + " (" + vj_compat::last_error() + ")");
}

struct db_hash_table {
    hash_t *hashes = nullptr;
    index_t size;
    bool gpu = false;
    bool data_owner = false;
    int device_index = 0;

    db_hash_table() {
        hashes = nullptr;
        size = 0;
        data_owner = true;
        device_index = 0;
    }
    db_hash_table(index_t table_size, bool gpu = true, int device_index = 0) {
        this->size = table_size;
        this->gpu = gpu;
        this->data_owner = true;
        this->device_index = device_index;
        if (gpu) {
            cudaSetDevice(device_index);
            if (cudaMalloc(&hashes, size * sizeof(hash_t)) != cudaSuccess) {
                hashes = nullptr;
            }
        } else {
            hashes = new hash_t[size];
        }
    }
    db_hash_table(index_t offset, index_t size, db_hash_table table_source) {
        this->size = size;
        this->gpu = table_source.gpu;
        this->hashes = &table_source.hashes[offset];
        this->data_owner = false;
        this->device_index = table_source.device_index;
    }
    int get_bytes() { return (int)(sizeof(hash_t) * size); }
    static int get_bytes(index_t size) { return (int)(sizeof(hash_t) * size); }
    void free() {
        if (data_owner) {
            if (gpu) {
                cudaSetDevice(device_index);
                cudaFree(hashes);
            } else {
                delete[] hashes;
            }
        }
        size = 0;
        hashes = nullptr;
    }
};

struct db_table {
    size_t column_count = 0;
    column_t *primary_keys = nullptr;
    column_t *column_values = nullptr;
    index_t size;
    bool gpu = false;
    bool data_owner = false;
    int device_index = 0;

    db_table() {
        column_count = 0;
        column_values = nullptr;
        primary_keys = nullptr;
        size = 0;
        data_owner = true;
        device_index = 0;
    }
    db_table(size_t column_count, index_t table_size, bool gpu = true) {
        this->column_count = column_count;
        this->size = table_size;
        this->gpu = gpu;
        this->data_owner = true;
        if (gpu) {
            if (cudaMalloc(&column_values, column_count * table_size * sizeof(column_t)) != cudaSuccess) column_values = nullptr;
            if (cudaMalloc(&primary_keys, table_size * sizeof(column_t)) != cudaSuccess) primary_keys = nullptr;
        } else {
            column_values = new column_t[column_count * table_size];
            primary_keys = new column_t[table_size];
        }
    }
    db_table(index_t offset, index_t size, db_table table_source) {
        this->device_index = table_source.device_index;
        this->size = size;
        this->gpu = table_source.gpu;
        this->column_count = table_source.column_count;
        this->data_owner = false;
        this->column_values = &table_source.column_values[offset * column_count];
        this->primary_keys = &table_source.primary_keys[offset];
    }
    db_table copy(bool to_gpu) {
        db_table t;
        t.column_count = column_count;
        t.gpu = to_gpu;
        t.data_owner = true;
        t.size = size;
        t.device_index = device_index;
        const size_t vb = size * column_count * sizeof(column_t), pb = size * sizeof(column_t);
        if (to_gpu) {
            cudaMalloc(&t.column_values, vb ? vb : 8);
            cudaMalloc(&t.primary_keys, pb ? pb : 8);
            cudaMemcpy(t.column_values, column_values, vb, gpu ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
            cudaMemcpy(t.primary_keys, primary_keys, pb, gpu ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
        } else {
            t.column_values = new column_t[size * column_count];
            t.primary_keys = new column_t[size];
            cudaMemcpy(t.column_values, column_values, vb, gpu ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
            cudaMemcpy(t.primary_keys, primary_keys, pb, gpu ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
        }
        return t;
    }
    int get_bytes() { return (int)get_bytes(size, (int)column_count); }
    static size_t get_bytes(index_t elements, int columns) { return sizeof(column_t) * elements * (columns + 1); }
    void free() { free(0); }
    void free(cudaStream_t stream) {
        if (size > 0) {
            if (data_owner) {
                if (gpu) {
                    cudaSetDevice(device_index);
                    if (stream) {
                        cudaFreeAsync(column_values, stream);
                        cudaFreeAsync(primary_keys, stream);
                    } else {
                        cudaFree(column_values);
                        cudaFree(primary_keys);
                    }
                } else {
                    delete[] column_values;
                    delete[] primary_keys;
                }
            }
            column_count = 0;
            size = 0;
            column_values = nullptr;
            primary_keys = nullptr;
        }
    }
    // vj view of the key columns (column_count u64 words pairs) and primary keys
    vj_table view() const {
        vj_table t;
        t.keys = column_values;
        t.payloads = primary_keys;
        t.rows = size;
        t.key_words = (int32_t)(2 * column_count);
        t.payload_bytes = 8;
        return t;
    }
};

// ---------------------------------------------------------------- hash (hash.cu:1-557)

struct HashSummary {
    std::string algorithm = "fnv";
    index_t elements = 0;
    int element_bytes = 0;
    int element_offset = 0;
    float k_tuples_p_seconds = 0.0;
    float k_gb_p_seconds = 0.0;
};

struct HashConfig {
    int threads_per_block = 256;
    int elements_per_thread = 1;
    std::string algorithm = "fnv";
    cudaStream_t stream = 0;
    bool profile_enabled = false;
    cudaEvent_t profile_start, profile_end;
    HashSummary profile_summary;
    int last_status = VJ_OK;

    void enable_profile(cudaEvent_t start, cudaEvent_t end) {
        profile_start = start;
        profile_end = end;
        profile_enabled = true;
    }
    void disbale_profile() { profile_enabled = false; }
};

inline void hash_func(index_t element_buffer_size, short int chunk_offset, short int element_chunks, chunk_t *element_buffer, hash_t *hashed_buffer, HashConfig &hash_config) {
    if (hash_config.profile_enabled) cudaEventRecord(hash_config.profile_start, hash_config.stream);
    const int algo = vj_hash_algo_id(hash_config.algorithm.c_str());
    hash_config.last_status = algo < 0 ? VJ_ERR_INVALID_ARGUMENT
                                       : vj_hash(element_buffer, element_buffer_size, chunk_offset, element_chunks, HASH_CHUNK_BITS, HASH_BITS, algo, hashed_buffer, (vj_stream_t)hash_config.stream);
    if (hash_config.profile_enabled) {
        cudaEventRecord(hash_config.profile_end, hash_config.stream);
        float ms = 0.f;
        cudaEventSynchronize(hash_config.profile_end);
        cudaEventElapsedTime(&ms, hash_config.profile_start, hash_config.profile_end);
        const float s = ms / 1e3f;
        HashSummary &p = hash_config.profile_summary;
        p.k_tuples_p_seconds = element_buffer_size / s;
        p.k_gb_p_seconds = (float)((element_chunks - chunk_offset) * sizeof(chunk_t)) * element_buffer_size / s / 1e9f;
        p.algorithm = hash_config.algorithm;
        p.elements = element_buffer_size;
        p.element_bytes = element_chunks * sizeof(chunk_t);
        p.element_offset = chunk_offset * sizeof(chunk_t);
    }
}

// ---------------------------------------------------------------- partition (cu:95-175, :610-661)

struct PartitionSummary {
    int device_index = 0;
    int stream_index = 0;
    int max_streams = 0;
    int buckets = 0;
    int depth = 0;
    size_t vector_bytes = 0;
    index_t elements = 0;
    std::string hash_function = "";
    float k_histogram_second = 0.0;
    float k_prefix_second = 0.0;
    float k_swap_second = 0.0;
    float k_histogram_elements_p_second = 0.0;
    float k_histogram_gb_p_second = 0.0;
    float k_swap_elements_p_second = 0.0;
    float k_swap_gb_p_second = 0.0;
};

struct PartitionConfig {
    int histogram_threads = 256;
    int histogram_n_elements_p_thread = 4;
    int swap_threads = 256;
    int swap_n_elements_p_thread = 1;
    int radix_width = 0;
    int bins = 0;
    index_t *d_histogram = nullptr;
    index_t *d_offsets = nullptr;
    index_t *d_dest_indices = nullptr;
    bool profiling_enabled = false;
    PartitionSummary profiling_summary;
    cudaEvent_t profiling_start, profiling_end;
    cudaStream_t stream = 0;
    int last_status = VJ_OK;

    void enable_profiling(cudaEvent_t start, cudaEvent_t end) {
        profiling_enabled = true;
        profiling_start = start;
        profiling_end = end;
    }
    void disable_profiling() { profiling_enabled = false; }
    void set_radix_width(int width) {
        radix_width = width;
        int new_bins = 1 << width;
        if (new_bins != bins) {
            free();
            bins = new_bins;
            cudaMallocAsync(&d_histogram, bins * sizeof(index_t), stream);
            cudaMallocAsync(&d_offsets, bins * sizeof(index_t), stream);
            cudaMallocAsync(&d_dest_indices, bins * sizeof(index_t), stream);
        }
    }
    void free() {
        if (d_dest_indices) cudaFreeAsync(d_dest_indices, stream);
        if (d_histogram) cudaFreeAsync(d_histogram, stream);
        if (d_offsets) cudaFreeAsync(d_offsets, stream);
        d_dest_indices = d_histogram = d_offsets = nullptr;
        bins = 0;
    }
};

inline void partition_gpu(db_table d_table, db_hash_table d_hash_table, db_table d_table_swap, db_hash_table d_hash_table_swap, int radix_shift, index_t *histogram, index_t *offsets,
                          PartitionConfig &partition_config) {
    partition_config.profiling_summary.elements = d_table.size;
    vj_table in = d_table.view();
    if (partition_config.profiling_enabled) cudaEventRecord(partition_config.profiling_start, partition_config.stream);
    partition_config.last_status =
        vj_partition(vj_compat::context(d_table.device_index), &in, d_hash_table.hashes, HASH_BITS, VJ_HASH_FNV, d_table_swap.column_values, d_table_swap.primary_keys, d_hash_table_swap.hashes, radix_shift,
                     partition_config.radix_width, (uint64_t *)partition_config.d_histogram, (uint64_t *)partition_config.d_offsets, (uint64_t *)histogram, (uint64_t *)offsets,
                     (vj_stream_t)partition_config.stream);
    if (partition_config.profiling_enabled) {
        cudaEventRecord(partition_config.profiling_end, partition_config.stream);
        float ms = 0.f;
        cudaEventSynchronize(partition_config.profiling_end);
        cudaEventElapsedTime(&ms, partition_config.profiling_start, partition_config.profiling_end);
        const float s = ms / 1e3f;
        partition_config.profiling_summary.k_swap_second = s;
        partition_config.profiling_summary.k_swap_elements_p_second = d_table.size / s;
        partition_config.profiling_summary.k_swap_gb_p_second = d_table.size * (sizeof(hash_t) + d_table.column_count * sizeof(column_t)) / s / 1e9f;
    }
}

// ---------------------------------------------------------------- build + probe (cu:177-287, :669-847)

struct ProbeSummary {
    int probe_mode = 0;
    index_t r_elements = 0;
    index_t s_elements = 0;
    index_t rs_elements = 0;
    float k_build_probe_tuples_p_second = 0.0;
    float k_build_probe_gb_p_second = 0.0;
    float k_extract_tuples_p_second = 0.0;
    float k_extract_gb_p_second = 0.0;
};

struct ProbeConfig {
    static const int MODE_PARTITION_R = 0;
    static const int MODE_PARTITION_S = 1;
    static const int MODE_GLOBAL_R = 2;
    int probe_mode = 0;
    float build_table_load = 0.75;
    int build_n_per_thread = 1;
    int build_threads = 256;
    int extract_n_per_thread = 1;
    int extract_threads = 256;
    int max_r_bytes = 48000;
    bool profiling_enabled = false;
    ProbeSummary profiling_summary;
    cudaEvent_t profiling_start, profiling_end;
    cudaStream_t stream = 0;

    void enable_profiling(cudaEvent_t start, cudaEvent_t end) {
        profiling_enabled = true;
        profiling_start = start;
        profiling_end = end;
    }
    void disable_profiling() { profiling_enabled = false; }
    void free() {}
};

// Allocates the rs table (column_count 2: [r_pk, s_pk] per row) of the pairs of r and s.
inline JoinStatus build_and_probe_gpu(db_table d_r_table, db_hash_table d_r_hash_table, db_table d_s_table, db_hash_table d_s_hash_table, db_table &d_joined_rs_table, int key_offset, ProbeConfig &config) {
    if (config.probe_mode < 0 || config.probe_mode > 2) {
        return JoinStatus(false, "Unknown probing mode");
    }
    vj_ctx *ctx = vj_compat::context(d_r_table.device_index);
    if (!ctx) return JoinStatus(false, "no vj context: " + vj_compat::last_error());
    vj_table r = d_r_table.view(), s = d_s_table.view();
    const void *rh = d_r_hash_table.hashes, *sh = d_s_hash_table.hashes;
    if (config.profiling_enabled) cudaEventRecord(config.profiling_start, config.stream);
    uint64_t cap = d_s_table.size ? d_s_table.size : 1;
    uint64_t count = 0;
    d_joined_rs_table = db_table();
    d_joined_rs_table.column_count = 2;
    d_joined_rs_table.gpu = true;
    d_joined_rs_table.data_owner = true;
    d_joined_rs_table.device_index = d_r_table.device_index;
    for (int attempt = 0; attempt < 2; attempt++) {
        column_t *pairs = nullptr;
        if (cudaMalloc(&pairs, cap * 2 * sizeof(column_t)) != cudaSuccess) {
            return JoinStatus(false, "Not enough memory for rs table");
        }
        int st = vj_build_probe(ctx, &r, rh, &s, sh, HASH_BITS, key_offset, pairs, cap, &count, (vj_stream_t)config.stream);
        if (st == VJ_OK) {
            d_joined_rs_table.column_values = pairs;
            break;
        }
        cudaFree(pairs);
        if (st != VJ_ERR_CAPACITY) return status_from(st, "build_and_probe_gpu");
        cap = count;
    }
    d_joined_rs_table.size = count;
    cudaMalloc(&d_joined_rs_table.primary_keys, (count ? count : 1) * sizeof(column_t));
    if (count) {
        std::vector<column_t> ids(count);
        for (uint64_t i = 0; i < count; i++) ids[i] = i + 1;
        cudaMemcpyAsync(d_joined_rs_table.primary_keys, ids.data(), count * sizeof(column_t), cudaMemcpyHostToDevice, config.stream);
        cudaStreamSynchronize(config.stream);
    }
    if (config.profiling_enabled) {
        cudaEventRecord(config.profiling_end, config.stream);
        cudaEventSynchronize(config.profiling_end);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, config.profiling_start, config.profiling_end);
        const float sec = ms / 1e3f;
        config.profiling_summary.k_build_probe_tuples_p_second = (d_r_table.size + d_s_table.size) / sec;
        config.profiling_summary.r_elements = d_r_table.size;
        config.profiling_summary.s_elements = d_s_table.size;
        config.profiling_summary.rs_elements = count;
    }
    return JoinStatus(true);
}

// ---------------------------------------------------------------- JoinProvider (cuh:54-429)

struct JoinSummary {
    JoinStatus join_status;
    float hash_tuples_p_second = 0.0;
    std::vector<HashSummary> hash_summaries;
    float partition_tuples_p_second = 0.0;
    std::vector<PartitionSummary> partition_summaries;
    float probe_tuples_p_second = 0.0;
    std::vector<ProbeSummary> probe_summaries;
    float merge_tuples_p_second = 0.0;
    float merge_gb_p_second = 0.0;
    float join_tuples_p_second = 0.0;
    float join_gb_p_second = 0.0;
    index_t r_elements = 0;
    index_t s_elements = 0;
    index_t rs_elements = 0;
};

struct JoinConfig {
    static const int MODE_RADIX_SPLIT = 0;
    static const int MODE_VECTOR_SPLIT = 1;
    int tasks_p_device = 1;
    int devices = 1;
    bool profile_enabled = true;
    int vector_bytes_size = 0;
    int join_mode = MODE_RADIX_SPLIT;
    int buckets = 2;
    HashConfig hash_config;
    PartitionConfig partition_config;
    ProbeConfig probe_config;
};

class JoinProvider {
  public:
    JoinProvider(JoinConfig join_config) : join_config(join_config) {}

    JoinStatus join(db_table r_table, db_table s_table, db_table &joined_rs_table) {
        if (r_table.gpu != s_table.gpu) {
            join_summary.join_status = JoinStatus(false, "Unable to figure out the join algorithm");
            return join_summary.join_status;
        }
        if (r_table.column_count != s_table.column_count) {
            join_summary.join_status = JoinStatus(false, "Tables differ in their key columns");
            return join_summary.join_status;
        }
        join_summary = JoinSummary();
        auto t0 = std::chrono::high_resolution_clock::now();
        vj_ctx *ctx = vj_compat::context(0);
        if (!ctx) return JoinStatus(false, "no vj context: " + vj_compat::last_error());
        vj_ctx_set_profiling(ctx, join_config.profile_enabled ? 1 : 0);
        vj_join_options opt;
        std::memset(&opt, 0, sizeof(opt));
        int algo = vj_hash_algo_id(join_config.hash_config.algorithm.c_str());
        opt.hash_algo = algo < 0 ? VJ_HASH_FNV : algo;
        opt.hash_bits = HASH_BITS;
        cudaStream_t stream = join_config.hash_config.stream;
        vj_table r = r_table.view(), s = s_table.view();
        uint64_t cap = s_table.size ? s_table.size : 1;
        uint64_t count = 0;
        JoinStatus status(true);
        joined_rs_table = db_table();
        joined_rs_table.column_count = 2;
        joined_rs_table.data_owner = true;
        joined_rs_table.gpu = r_table.gpu;
        for (int attempt = 0; attempt < 2; attempt++) {
            column_t *pairs = nullptr;
            int st;
            if (r_table.gpu) {
                if (cudaMalloc(&pairs, cap * 2 * sizeof(column_t)) != cudaSuccess) return fail(JoinStatus(false, "Not enough memory for rs table"));
                vj_result res;
                std::memset(&res, 0, sizeof(res));
                res.pairs = pairs;
                res.capacity = cap;
                st = vj_join(ctx, &r, &s, &opt, &res, (vj_stream_t)stream);
                count = res.count;
                if (st != VJ_OK) cudaFree(pairs);
            } else {
                pairs = new column_t[cap * 2];
                st = vj_join_host(ctx, &r, &s, &opt, pairs, cap, &count, (vj_stream_t)stream);
                if (st != VJ_OK) delete[] pairs;
            }
            if (st == VJ_OK) {
                joined_rs_table.column_values = pairs;
                break;
            }
            if (st != VJ_ERR_CAPACITY) return fail(status_from(st, "join"));
            cap = count;
        }
        joined_rs_table.size = count;
        if (r_table.gpu) {
            cudaMalloc(&joined_rs_table.primary_keys, (count ? count : 1) * sizeof(column_t));
            std::vector<column_t> ids(count);
            for (uint64_t i = 0; i < count; i++) ids[i] = i + 1;
            if (count) cudaMemcpy(joined_rs_table.primary_keys, ids.data(), count * sizeof(column_t), cudaMemcpyHostToDevice);
        } else {
            joined_rs_table.primary_keys = new column_t[count ? count : 1];
            for (uint64_t i = 0; i < count; i++) joined_rs_table.primary_keys[i] = i + 1;
        }
        auto t1 = std::chrono::high_resolution_clock::now();
        const double sec = std::chrono::duration<double>(t1 - t0).count();
        const double tuples = (double)(r_table.size + s_table.size);
        vj_profile prof;
        std::memset(&prof, 0, sizeof(prof));
        vj_ctx_last_profile(ctx, &prof);
        auto rate = [&](float ms) { return ms > 0.f ? (float)(tuples / (ms / 1e3)) : 0.f; };
        join_summary.partition_tuples_p_second = rate(prof.ms_histogram[0] + prof.ms_histogram[1] + prof.ms_scatter[0] + prof.ms_scatter[1] + prof.ms_plan[0] + prof.ms_plan[1]);
        join_summary.probe_tuples_p_second = rate(prof.ms_probe);
        join_summary.join_tuples_p_second = (float)(tuples / sec);
        join_summary.join_gb_p_second = (float)(tuples * r_table.column_count * sizeof(column_t) / 1e9 / sec);
        join_summary.rs_elements = count;
        join_summary.r_elements = r_table.size;
        join_summary.s_elements = s_table.size;
        join_summary.join_status = status;
        return status;
    }

    JoinSummary get_join_summary() { return join_summary; }

  private:
    JoinStatus fail(JoinStatus s) {
        join_summary.join_status = s;
        return s;
    }
    JoinConfig join_config;
    JoinSummary join_summary;
};
