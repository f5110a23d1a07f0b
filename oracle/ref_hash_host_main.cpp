/*
 * Tail appended after the reference's hash kernels (src/hash/hash.cu:1-505, with the
 * dispatcher hash_func at :507-557 left out because it uses the <<<>>> launch syntax) by
 * oracle/ref_build.sh. Test infrastructure only.
 *
 * usage: ref_hash_host <algorithm name> <n> <chunk_offset> <element_chunks> <in.bin> <out.bin>
 * Calls the reference kernel named like the dispatcher does (hash.cu:515-541, rounds = 2
 * for custom_n_mult_xor_shift) and writes n hash_t values.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

int main(int argc, char **argv) {
    if (argc != 7) {
        fprintf(stderr, "usage: %s algo n chunk_offset element_chunks in out\n", argv[0]);
        return 2;
    }
    std::string algo = argv[1];
    index_t n = strtoull(argv[2], nullptr, 10);
    short chunk_offset = (short)atoi(argv[3]);
    short element_chunks = (short)atoi(argv[4]);
    size_t in_bytes = (size_t)n * element_chunks * sizeof(chunk_t);
    std::vector<unsigned char> in(in_bytes + 16);
    FILE *f = fopen(argv[5], "rb");
    if (!f || fread(in.data(), 1, in_bytes, f) != in_bytes) {
        fprintf(stderr, "cannot read %s\n", argv[5]);
        return 3;
    }
    fclose(f);
    std::vector<hash_t> out(n + 1);
    chunk_t *buf = (chunk_t *)in.data();
    hash_t *h = out.data();
    if (algo == "fnv") hash_fnv(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_xor") hash_custom_xor(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_xor_shift") hash_custom_xor_shift(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_xor_hw") hash_custom_xor_hw(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_mult_xor_shift") hash_custom_mult_xor_shift(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_n_mult_xor_shift") hash_custom_n_mult_xor_shift(n, chunk_offset, element_chunks, 2, buf, h);
    else if (algo == "custom_mult_xor_hw") hash_custom_mult_xor_hw(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_mult") hash_custom_mult(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_mult_shift") hash_custom_mult_shift(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_mult_hw") hash_custom_mult_hw(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_add") hash_custom_add(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_add_shift") hash_custom_add_shift(n, chunk_offset, element_chunks, buf, h);
    else if (algo == "custom_add_hw") hash_custom_add_hw(n, chunk_offset, element_chunks, buf, h);
    else {
        fprintf(stderr, "unknown algorithm %s\n", algo.c_str());
        return 4;
    }
    f = fopen(argv[6], "wb");
    if (!f || fwrite(h, sizeof(hash_t), n, f) != n) {
        fprintf(stderr, "cannot write %s\n", argv[6]);
        return 5;
    }
    fclose(f);
    return 0;
}
