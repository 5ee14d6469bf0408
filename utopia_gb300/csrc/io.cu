// On-disk operators and vectors: PETSc binary and raw CRS files.
//
// The reference reads its inputs with utopia::read (PETSc MatLoad / VecLoad for the PETSc binary
// files of utopia/data, e.g. utopia/apps/ls_solve/utopia_ls_solve.cpp:117-133) and raw CRS
// arrays (rowptr.raw, colidx.raw, values.raw of one directory; utopia/data/test/qpsolve.yaml:13-35).
// PETSc binary layout (big endian, 32-bit indices): Mat = int32 classid 1211216, M, N, nnz,
// row lengths[M], column indices[nnz], float64 values[nnz]; Vec = int32 classid 1211214, N,
// float64 values[N].  Raw CRS: native-endian arrays, rowptr[n + 1] and colidx[nnz] of
// index_bytes (4 or 8) each, values[nnz] of value_bytes (8 or 4) each.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "abi_util.cuh"
#include "device_util.cuh"

namespace {

using ugpu::Error;

constexpr int32_t kPetscMatId = 1211216;
constexpr int32_t kPetscVecId = 1211214;

std::vector<unsigned char> slurp(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    UGPU_CHECK(f, UGPU_ERR_ARG, "cannot open " + path);
    std::vector<unsigned char> buf;
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
    return buf;
}

void spill(const std::string &path, const std::vector<unsigned char> &buf) {
    FILE *f = std::fopen(path.c_str(), "wb");
    UGPU_CHECK(f, UGPU_ERR_ARG, "cannot create " + path);
    const size_t put = buf.empty() ? 0 : std::fwrite(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    UGPU_CHECK(put == buf.size(), UGPU_ERR_ARG, "short write to " + path);
}

// big-endian fields
struct BeReader {
    const std::vector<unsigned char> &b;
    size_t pos = 0;
    const std::string &path;
    uint64_t take(int bytes) {
        UGPU_CHECK(pos + size_t(bytes) <= b.size(), UGPU_ERR_ARG, "truncated PETSc binary file " + path);
        uint64_t v = 0;
        for (int i = 0; i < bytes; ++i) v = (v << 8) | b[pos + size_t(i)];
        pos += size_t(bytes);
        return v;
    }
    int32_t i32() { return int32_t(uint32_t(take(4))); }
    double f64() {
        const uint64_t u = take(8);
        double d;
        std::memcpy(&d, &u, 8);
        return d;
    }
};

void put_be(std::vector<unsigned char> &out, uint64_t v, int bytes) {
    for (int i = bytes - 1; i >= 0; --i) out.push_back(static_cast<unsigned char>((v >> (8 * i)) & 0xffu));
}
void put_i32(std::vector<unsigned char> &out, int32_t v) { put_be(out, uint32_t(v), 4); }
void put_f64(std::vector<unsigned char> &out, double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    put_be(out, u, 8);
}

template <class T>
std::vector<T> native_array(const std::string &path, int bytes, const char *what) {
    auto raw = slurp(path);
    UGPU_CHECK(raw.size() % size_t(bytes) == 0, UGPU_ERR_ARG, std::string(what) + ": size of " + path +
                                                                  " is not a multiple of the element size");
    const size_t n = raw.size() / size_t(bytes);
    std::vector<T> out(n);
    for (size_t i = 0; i < n; ++i) {
        if (bytes == 8) {
            if constexpr (std::is_floating_point<T>::value) {
                double d;
                std::memcpy(&d, raw.data() + 8 * i, 8);
                out[i] = T(d);
            } else {
                int64_t q;
                std::memcpy(&q, raw.data() + 8 * i, 8);
                out[i] = T(q);
            }
        } else {
            if constexpr (std::is_floating_point<T>::value) {
                float d;
                std::memcpy(&d, raw.data() + 4 * i, 4);
                out[i] = T(d);
            } else {
                int32_t q;
                std::memcpy(&q, raw.data() + 4 * i, 4);
                out[i] = T(q);
            }
        }
    }
    return out;
}

std::string join(const std::string &dir, const char *name) {
    return dir.empty() || dir.back() == '/' ? dir + name : dir + "/" + name;
}

}  // namespace

extern "C" {

int ugpu_petsc_read_mat(ugpu_ctx *ctx, const char *path, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_REQUIRE(path);
    const std::string p(path);
    auto buf = slurp(p);
    BeReader r{buf, 0, p};
    UGPU_CHECK(r.i32() == kPetscMatId, UGPU_ERR_ARG, p + " is not a PETSc binary matrix");
    const int32_t M = r.i32(), N = r.i32(), nz = r.i32();
    UGPU_CHECK(M >= 0 && N >= 0 && nz >= 0, UGPU_ERR_UNSUPPORTED,
               p + ": dense or special PETSc matrix layouts are not supported");
    std::vector<int32_t> rp(size_t(M) + 1, 0), ci(static_cast<size_t>(nz));
    std::vector<double> v(static_cast<size_t>(nz));
    for (int32_t i = 0; i < M; ++i) {
        const int32_t len = r.i32();
        UGPU_CHECK(len >= 0, UGPU_ERR_ARG, p + ": negative row length");
        rp[size_t(i) + 1] = rp[size_t(i)] + len;
    }
    UGPU_CHECK(rp[size_t(M)] == nz, UGPU_ERR_ARG, p + ": row lengths do not add up to nnz");
    for (auto &c : ci) c = r.i32();
    for (auto &x : v) x = r.f64();
    const int rc = ugpu_csr_create(ctx, M, N, nz, rp.data(), ci.data(), v.data(), out);
    if (rc != UGPU_OK) return rc;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_petsc_read_vec(ugpu_ctx *ctx, const char *path, ugpu_vec **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_REQUIRE(path);
    const std::string p(path);
    auto buf = slurp(p);
    BeReader r{buf, 0, p};
    UGPU_CHECK(r.i32() == kPetscVecId, UGPU_ERR_ARG, p + " is not a PETSc binary vector");
    const int32_t n = r.i32();
    UGPU_CHECK(n >= 0, UGPU_ERR_ARG, p + ": negative size");
    std::vector<double> v(static_cast<size_t>(n));
    for (auto &x : v) x = r.f64();
    int rc = ugpu_vec_create(ctx, n, UGPU_F64, out);
    if (rc == UGPU_OK) rc = ugpu_vec_upload(*out, v.data());
    if (rc != UGPU_OK) return rc;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_petsc_write_mat(const ugpu_mat *A, const char *path) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(path);
    const auto &M = A->impl;
    UGPU_CHECK(M.nrows < (1ll << 31) && M.ncols < (1ll << 31), UGPU_ERR_UNSUPPORTED, "PETSc binary: 32-bit sizes");
    std::vector<int32_t> rp(size_t(M.nrows) + 1), ci(size_t(M.nnz));
    std::vector<double> v(size_t(M.nnz));
    const int rc = ugpu_csr_download(A, rp.data(), ci.data(), v.data());
    if (rc != UGPU_OK) return rc;
    std::vector<unsigned char> out;
    out.reserve(16 + 4 * rp.size() + 12 * v.size());
    put_i32(out, kPetscMatId);
    put_i32(out, int32_t(M.nrows));
    put_i32(out, int32_t(M.ncols));
    put_i32(out, int32_t(M.nnz));
    for (int64_t i = 0; i < M.nrows; ++i) put_i32(out, rp[size_t(i) + 1] - rp[size_t(i)]);
    for (int32_t c : ci) put_i32(out, c);
    for (double x : v) put_f64(out, x);
    spill(path, out);
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_petsc_write_vec(const ugpu_vec *x, const char *path) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(path);
    UGPU_CHECK(x->impl.dtype == UGPU_F64, UGPU_ERR_ARG, "PETSc binary: FP64 vector required");
    std::vector<double> v(size_t(x->impl.n));
    const int rc = ugpu_vec_download(x, v.data());
    if (rc != UGPU_OK) return rc;
    std::vector<unsigned char> out;
    put_i32(out, kPetscVecId);
    put_i32(out, int32_t(x->impl.n));
    for (double d : v) put_f64(out, d);
    spill(path, out);
    UGPU_ABI_END(x ? x->impl.ctx : nullptr)
}

int ugpu_raw_crs_read(ugpu_ctx *ctx, const char *dir, int index_bytes, int value_bytes, int64_t ncols,
                      ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_REQUIRE(dir);
    UGPU_CHECK(index_bytes == 4 || index_bytes == 8, UGPU_ERR_ARG, "raw CRS: index_bytes must be 4 or 8");
    UGPU_CHECK(value_bytes == 4 || value_bytes == 8, UGPU_ERR_ARG, "raw CRS: value_bytes must be 4 or 8");
    const std::string d(dir);
    auto rp64 = native_array<int64_t>(join(d, "rowptr.raw"), index_bytes, "raw CRS rowptr");
    auto ci64 = native_array<int64_t>(join(d, "colidx.raw"), index_bytes, "raw CRS colidx");
    auto v = native_array<double>(join(d, "values.raw"), value_bytes, "raw CRS values");
    UGPU_CHECK(!rp64.empty(), UGPU_ERR_ARG, "raw CRS: empty rowptr");
    const int64_t n = int64_t(rp64.size()) - 1, nnz = int64_t(ci64.size());
    UGPU_CHECK(rp64.front() == 0 && rp64.back() == nnz && int64_t(v.size()) == nnz, UGPU_ERR_ARG,
               "raw CRS: rowptr, colidx and values disagree on the number of entries");
    UGPU_CHECK(nnz < (1ll << 31) && n < (1ll << 31), UGPU_ERR_UNSUPPORTED, "raw CRS: more than 2^31 entries");
    std::vector<int32_t> rp(rp64.begin(), rp64.end()), ci(ci64.begin(), ci64.end());
    const int64_t m = ncols > 0 ? ncols : n;  // square unless given
    const int rc = ugpu_csr_create(ctx, n, m, nnz, rp.data(), ci.data(), v.data(), out);
    if (rc != UGPU_OK) return rc;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_raw_vec_read(ugpu_ctx *ctx, const char *path, int value_bytes, ugpu_vec **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_REQUIRE(path);
    UGPU_CHECK(value_bytes == 4 || value_bytes == 8, UGPU_ERR_ARG, "raw vector: value_bytes must be 4 or 8");
    auto v = native_array<double>(path, value_bytes, "raw vector");
    int rc = ugpu_vec_create(ctx, int64_t(v.size()), UGPU_F64, out);
    if (rc == UGPU_OK) rc = ugpu_vec_upload(*out, v.data());
    if (rc != UGPU_OK) return rc;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_raw_vec_write(const ugpu_vec *x, const char *path) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(path);
    UGPU_CHECK(x->impl.dtype == UGPU_F64, UGPU_ERR_ARG, "raw vector: FP64 vector required");
    std::vector<double> v(size_t(x->impl.n));
    const int rc = ugpu_vec_download(x, v.data());
    if (rc != UGPU_OK) return rc;
    std::vector<unsigned char> out(v.size() * 8);
    if (!v.empty()) std::memcpy(out.data(), v.data(), out.size());
    spill(path, out);
    UGPU_ABI_END(x ? x->impl.ctx : nullptr)
}

}  // extern "C"
