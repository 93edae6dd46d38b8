// archive.hpp -- the byte layout of seqan::hibf's serialised filters (cereal's binary archive encoding of the
// reference's serialize functions: interleaved_bloom_filter.hpp:471-485, bit_vector.hpp:885-925,
// hierarchical_interleaved_bloom_filter.hpp:267-277), read and written straight from and to the device stores.
//
// Encoding: arithmetic values as their little-endian bytes (bool: one byte), a std::vector as a uint64 element count
// followed by its elements, name-value pairs as their value, a base class as the base object.
//   interleaved_bloom_filter: u32 version (1); u64 bins, technical_bins, bin_size, hash_shift, bin_words, hash_funs;
//     bit_vector: u64 size in bits, then ceil(bits / 64) u64 words (row-major, bin_words per row);
//     occupancy: u64 count (technical_bins), u64 each; u8 track_occupancy.
//   hierarchical_interleaved_bloom_filter: u32 version (1); u64 number_of_user_bins; u64 count + each IBF;
//     next_ibf_id: u64 count + per IBF (u64 count + u64 each); prev_ibf_id: u64 count + (u64 ibf, u64 bin) each;
//     ibf_bin_to_user_bin_id: as next_ibf_id.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "common.hpp"

namespace hibf_gb300
{

constexpr uint32_t kArchiveVersion = 1;

class file_writer
{
public:
    explicit file_writer(char const * path) : f_{std::fopen(path, "wb")}
    {
        if (!f_)
            fail(HIBF_GPU_ERR_INVALID_ARG, std::string("cannot open for writing: ") + path);
    }
    ~file_writer()
    {
        if (f_)
            std::fclose(f_);
    }
    file_writer(file_writer const &) = delete;
    file_writer & operator=(file_writer const &) = delete;

    void raw(void const * p, size_t n)
    {
        if (n && std::fwrite(p, 1, n, f_) != n)
            fail(HIBF_GPU_ERR_INVALID_ARG, "write failed");
    }
    void u8(uint8_t x)
    {
        raw(&x, 1);
    }
    void u32(uint32_t x)
    {
        raw(&x, 4);
    }
    void u64(uint64_t x)
    {
        raw(&x, 8);
    }
    void u64s(std::vector<uint64_t> const & v)
    {
        u64(v.size());
        raw(v.data(), v.size() * 8);
    }
    void close()
    {
        if (std::fclose(f_) != 0)
        {
            f_ = nullptr;
            fail(HIBF_GPU_ERR_INVALID_ARG, "write failed");
        }
        f_ = nullptr;
    }

private:
    std::FILE * f_;
};

class file_reader
{
public:
    explicit file_reader(char const * path) : f_{std::fopen(path, "rb")}
    {
        if (!f_)
            fail(HIBF_GPU_ERR_INVALID_ARG, std::string("cannot open: ") + path);
    }
    ~file_reader()
    {
        if (f_)
            std::fclose(f_);
    }
    file_reader(file_reader const &) = delete;
    file_reader & operator=(file_reader const &) = delete;

    void raw(void * p, size_t n)
    {
        if (n && std::fread(p, 1, n, f_) != n)
            fail(HIBF_GPU_ERR_INVALID_ARG, "archive truncated");
    }
    uint8_t u8()
    {
        uint8_t x{};
        raw(&x, 1);
        return x;
    }
    uint32_t u32()
    {
        uint32_t x{};
        raw(&x, 4);
        return x;
    }
    uint64_t u64()
    {
        uint64_t x{};
        raw(&x, 8);
        return x;
    }
    std::vector<uint64_t> u64s(uint64_t max_count)
    {
        uint64_t const n = u64();
        if (n > max_count)
            fail(HIBF_GPU_ERR_INVALID_ARG, "archive: implausible vector length");
        std::vector<uint64_t> v(n);
        raw(v.data(), n * 8);
        return v;
    }
    void skip(uint64_t n)
    {
        if (n && std::fseek(f_, static_cast<long>(n), SEEK_CUR) != 0)
            fail(HIBF_GPU_ERR_INVALID_ARG, "archive truncated");
    }
    long tell() const
    {
        return std::ftell(f_);
    }
    void seek(long pos)
    {
        if (std::fseek(f_, pos, SEEK_SET) != 0)
            fail(HIBF_GPU_ERR_INVALID_ARG, "seek failed");
    }
    bool at_end()
    {
        int const c = std::fgetc(f_);
        if (c == EOF)
            return true;
        std::ungetc(c, f_);
        return false;
    }

private:
    std::FILE * f_;
};

// The fields of one serialised IBF before its words.
struct ibf_header
{
    uint64_t bins, technical_bins, bin_size, hash_shift, bin_words, hash_funs, bits;
};

inline ibf_header read_ibf_header(file_reader & r)
{
    uint32_t const version = r.u32();
    if (version != kArchiveVersion)
        fail(HIBF_GPU_ERR_INVALID_ARG, "archive: unsupported interleaved_bloom_filter version");
    ibf_header h{};
    h.bins = r.u64();
    h.technical_bins = r.u64();
    h.bin_size = r.u64();
    h.hash_shift = r.u64();
    h.bin_words = r.u64();
    h.hash_funs = r.u64();
    h.bits = r.u64();
    if (h.bins == 0 || h.bin_size == 0 || h.hash_funs == 0 || h.hash_funs > 5 ||
        h.technical_bins != ((h.bins + 63) / 64) * 64 || h.bin_words != h.technical_bins / 64 ||
        h.bits != h.bin_size * h.technical_bins || h.hash_shift != static_cast<uint64_t>(__builtin_clzll(h.bin_size)))
        fail(HIBF_GPU_ERR_INVALID_ARG, "archive: inconsistent interleaved_bloom_filter fields");
    return h;
}

inline void write_ibf_header(file_writer & w, uint64_t bins, uint64_t bin_size, uint64_t hash_funs)
{
    uint64_t const tb = ((bins + 63) / 64) * 64;
    w.u32(kArchiveVersion);
    w.u64(bins);
    w.u64(tb);
    w.u64(bin_size);
    w.u64(static_cast<uint64_t>(__builtin_clzll(bin_size)));
    w.u64(tb / 64);
    w.u64(hash_funs);
    w.u64(bin_size * tb);
}

// Streams a device store of `rows` rows (row_words words apart, bin_words of them serialised) through a pinned
// host chunk into / out of the archive.
inline void write_rows(file_writer & w, uint64_t const * d_store, uint64_t rows, uint64_t bin_words,
                       uint64_t row_words, cudaStream_t s)
{
    uint64_t const rows_per_chunk = std::max<uint64_t>(1, (32ull << 20) / (bin_words * 8));
    hbuf chunk;
    chunk.ensure(std::min(rows, rows_per_chunk) * bin_words * 8);
    for (uint64_t r = 0; r < rows; r += rows_per_chunk)
    {
        uint64_t const n = std::min(rows_per_chunk, rows - r);
        HG_CUDA(cudaMemcpy2DAsync(chunk.p, bin_words * 8, d_store + r * row_words, row_words * 8, bin_words * 8, n,
                                  cudaMemcpyDeviceToHost, s));
        HG_CUDA(cudaStreamSynchronize(s));
        w.raw(chunk.p, n * bin_words * 8);
    }
}

inline void read_rows(file_reader & rd, uint64_t * d_store, uint64_t rows, uint64_t bin_words, uint64_t row_words,
                      cudaStream_t s)
{
    uint64_t const rows_per_chunk = std::max<uint64_t>(1, (32ull << 20) / (bin_words * 8));
    hbuf chunk;
    chunk.ensure(std::min(rows, rows_per_chunk) * bin_words * 8);
    for (uint64_t r = 0; r < rows; r += rows_per_chunk)
    {
        uint64_t const n = std::min(rows_per_chunk, rows - r);
        rd.raw(chunk.p, n * bin_words * 8);
        HG_CUDA(cudaMemcpy2DAsync(d_store + r * row_words, row_words * 8, chunk.p, bin_words * 8, bin_words * 8, n,
                                  cudaMemcpyHostToDevice, s));
        HG_CUDA(cudaStreamSynchronize(s));
    }
}

} // namespace hibf_gb300
