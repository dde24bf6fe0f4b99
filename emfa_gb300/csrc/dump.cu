// Binary dump format for matrices, vectors and operator arrays, in place of
// the reference's Armadillo ASCII dumps (EFIE::writeZIVData,
// EMSolver/EFIE.cpp:932-950; CFIE.cpp:797-812).  Used for golden vectors and
// for warm restarts of served problems.
//
// Layout (little-endian), 128-byte header then the payload, row-major:
//   0   char[8]  "EMFADUMP"
//   8   u32      format version (1)
//   12  u32      dtype: 1 complex64, 2 complex128, 3 float32, 4 float64, 5 int32
//   16  u64      rows
//   24  u64      cols
//   32  f64      frequency (Hz; 0 if not applicable)
//   40  char[24] name ("Z", "V", "I", ...), NUL-padded
//   64  u64      payload bytes (rows x cols x element size)
//   72  u64      FNV-1a 64-bit hash of the payload
//   80  zeros up to 128
#include "emfa_internal.cuh"

#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr char MAGIC[8] = {'E', 'M', 'F', 'A', 'D', 'U', 'M', 'P'};
constexpr uint32_t VERSION = 1;
constexpr size_t HEADER = 128;

size_t elem_bytes(int dtype)
{
    switch (dtype) {
        case 1: return 8;
        case 2: return 16;
        case 3: return 4;
        case 4: return 8;
        case 5: return 4;
        default: return 0;
    }
}

uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h = 1469598103934665603ull)
{
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

struct Header {
    char magic[8];
    uint32_t version, dtype;
    uint64_t rows, cols;
    double freq;
    char name[24];
    uint64_t bytes, hash;
    unsigned char pad[HEADER - 80];
};
static_assert(sizeof(Header) == HEADER, "dump header is 128 bytes");

emfa_status_t fail(const std::string& m, emfa_status_t s)
{
    emfa::set_error(nullptr, m);
    return s;
}

emfa_status_t read_header(FILE* f, Header* h, const char* path)
{
    if (std::fread(h, 1, HEADER, f) != HEADER) return fail(std::string("emfa_dump: short header in ") + path, EMFA_ERR_INVALID);
    if (std::memcmp(h->magic, MAGIC, 8) != 0) return fail(std::string("emfa_dump: not an EMFA dump: ") + path, EMFA_ERR_INVALID);
    if (h->version != VERSION)
        return fail("emfa_dump: unsupported format version " + std::to_string(h->version), EMFA_ERR_UNSUPPORTED);
    const size_t es = elem_bytes((int)h->dtype);
    if (!es || h->bytes != h->rows * h->cols * es) return fail("emfa_dump: inconsistent header", EMFA_ERR_INVALID);
    return EMFA_OK;
}

}  // namespace

extern "C" {

emfa_status_t emfa_dump_save(const char* path, const char* name, int dtype, size_t rows, size_t cols, double freq,
                             const void* data, int data_on_device)
{
    const size_t es = elem_bytes(dtype);
    if (!path || !data || !es || rows == 0 || cols == 0) return fail("emfa_dump_save: bad arguments", EMFA_ERR_INVALID);
    const size_t bytes = rows * cols * es;
    std::vector<unsigned char> host;
    const unsigned char* src = static_cast<const unsigned char*>(data);
    if (data_on_device) {
        host.resize(bytes);
        cudaError_t e = cudaMemcpy(host.data(), data, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(std::string("emfa_dump_save: ") + cudaGetErrorString(e), EMFA_ERR_CUDA);
        src = host.data();
    }
    Header h{};
    std::memcpy(h.magic, MAGIC, 8);
    h.version = VERSION;
    h.dtype = (uint32_t)dtype;
    h.rows = rows;
    h.cols = cols;
    h.freq = freq;
    if (name) std::strncpy(h.name, name, sizeof h.name - 1);
    h.bytes = bytes;
    h.hash = fnv1a(src, bytes);
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(std::string("emfa_dump_save: cannot open ") + path, EMFA_ERR_INVALID);
    const bool ok = std::fwrite(&h, 1, HEADER, f) == HEADER && std::fwrite(src, 1, bytes, f) == bytes;
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) return fail(std::string("emfa_dump_save: write failed: ") + path, EMFA_ERR_INVALID);
    return EMFA_OK;
}

emfa_status_t emfa_dump_info(const char* path, char* name_out, int* dtype, size_t* rows, size_t* cols, double* freq)
{
    if (!path) return fail("emfa_dump_info: bad arguments", EMFA_ERR_INVALID);
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(std::string("emfa_dump_info: cannot open ") + path, EMFA_ERR_INVALID);
    Header h{};
    const emfa_status_t s = read_header(f, &h, path);
    std::fclose(f);
    if (s != EMFA_OK) return s;
    if (name_out) {
        std::memcpy(name_out, h.name, sizeof h.name);
        name_out[sizeof h.name - 1] = 0;
    }
    if (dtype) *dtype = (int)h.dtype;
    if (rows) *rows = h.rows;
    if (cols) *cols = h.cols;
    if (freq) *freq = h.freq;
    return EMFA_OK;
}

emfa_status_t emfa_dump_load(const char* path, void* data, size_t capacity_bytes, int data_on_device)
{
    if (!path || !data) return fail("emfa_dump_load: bad arguments", EMFA_ERR_INVALID);
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(std::string("emfa_dump_load: cannot open ") + path, EMFA_ERR_INVALID);
    Header h{};
    emfa_status_t s = read_header(f, &h, path);
    if (s != EMFA_OK) {
        std::fclose(f);
        return s;
    }
    if (h.bytes > capacity_bytes) {
        std::fclose(f);
        return fail("emfa_dump_load: destination holds " + std::to_string(capacity_bytes) + " bytes, the dump " +
                        std::to_string(h.bytes),
                    EMFA_ERR_INVALID);
    }
    std::vector<unsigned char> host(h.bytes);
    const bool ok = std::fread(host.data(), 1, h.bytes, f) == h.bytes;
    std::fclose(f);
    if (!ok) return fail(std::string("emfa_dump_load: truncated payload in ") + path, EMFA_ERR_INVALID);
    if (fnv1a(host.data(), h.bytes) != h.hash)
        return fail(std::string("emfa_dump_load: payload hash mismatch (corrupted file): ") + path, EMFA_ERR_INVALID);
    if (data_on_device) {
        cudaError_t e = cudaMemcpy(data, host.data(), h.bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(std::string("emfa_dump_load: ") + cudaGetErrorString(e), EMFA_ERR_CUDA);
    } else {
        std::memcpy(data, host.data(), h.bytes);
    }
    return EMFA_OK;
}

}  // extern "C"
