// Binary CSR / vector files in the reference's interchange format (the files its solver test reads
// and its time steppers dump: cpp/libs/LinAlg/src/io.cpp:49-148), so that a system written by the
// reference can be solved here and the other way round.
//
// Layout (native byte order, 4-byte ints):
//   CSR:    int dtype (0 float, 1 double), int rows, int cols, int nnz,
//           values[nnz] (dtype), column[nnz] (int), rowStart[rows + 1] (int)
//   vector: int dtype, int n, values[n] (dtype)
// Reading checks what the reference's reader checks (the dtype id, positive sizes, complete data,
// rowStart[rows] == nnz) and, in addition, that the CSR is well formed (validCsr), since the device
// operators rely on it.
#include "setup.hpp"

#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>

namespace nsf
{
    namespace
    {
        struct File
        {
            std::FILE * f = nullptr;
            File(const std::string & path, const char * mode) : f(std::fopen(path.c_str(), mode)) {}
            ~File()
            {
                if (f)
                    std::fclose(f);
            }
        };

        template <typename T>
        bool readN(std::FILE * f, T * dst, size_t n)
        {
            return n == 0 || std::fread(dst, sizeof(T), n, f) == n;
        }

        template <typename T>
        void writeN(std::FILE * f, const T * src, size_t n, const std::string & path)
        {
            if (n && std::fwrite(src, sizeof(T), n, f) != n)
                throw std::runtime_error("failed to write " + path);
        }

        void readValues(std::FILE * f, int dtype, size_t n, std::vector<double> & out, const char * what)
        {
            out.resize(n);
            if (dtype == 1)
            {
                if (!readN(f, out.data(), n))
                    throw std::runtime_error(std::string("failed to read ") + what + ": couldn't read data vectors");
                return;
            }
            std::vector<float> tmp(n);
            if (!readN(f, tmp.data(), n))
                throw std::runtime_error(std::string("failed to read ") + what + ": couldn't read data vectors");
            for (size_t i = 0; i < n; i++)
                out[i] = tmp[i];
        }

        void writeValues(std::FILE * f, int dtype, const double * v, size_t n, const std::string & path)
        {
            if (dtype == 1)
            {
                writeN(f, v, n, path);
                return;
            }
            std::vector<float> tmp(v, v + n);
            writeN(f, tmp.data(), n, path);
        }
    } // namespace

    BinCsr readBinCsr(const std::string & path)
    {
        File F(path, "rb");
        if (!F.f)
            throw std::runtime_error("failed to open input file " + path);
        int hdr[4];
        if (!readN(F.f, hdr, 1) || (hdr[0] != 0 && hdr[0] != 1))
            throw std::runtime_error("failed to read CSR matrix: bad dtype");
        if (!readN(F.f, hdr + 1, 3))
            throw std::runtime_error("failed to read CSR matrix: couldn't read header");
        BinCsr m;
        m.dtype = hdr[0];
        m.a.rows = hdr[1];
        m.a.cols = hdr[2];
        const int nnz = hdr[3];
        if (m.a.rows < 1 || m.a.cols < 1 || nnz < 1)
            throw std::runtime_error("failed to read CSR matrix: bad header values");
        readValues(F.f, m.dtype, (size_t)nnz, m.a.val, "CSR matrix");
        m.a.col.resize(nnz);
        m.a.rowStart.resize((size_t)m.a.rows + 1);
        if (!readN(F.f, m.a.col.data(), (size_t)nnz) || !readN(F.f, m.a.rowStart.data(), (size_t)m.a.rows + 1))
            throw std::runtime_error("failed to read CSR matrix: couldn't read data vectors");
        if (m.a.rowStart.back() != nnz)
            throw std::runtime_error("failed to read CSR matrix: bad end of rowStart");
        std::string why;
        if (!validCsr(m.a.rows, m.a.cols, nnz, m.a.rowStart.data(), m.a.col.data(), why))
            throw std::runtime_error("failed to read CSR matrix: " + why);
        return m;
    }

    void writeBinCsr(const std::string & path, int rows, int cols, int nnz, const int * rowStart, const int * col,
                     const double * values, int dtype)
    {
        if (dtype != 0 && dtype != 1)
            throw std::invalid_argument("dtype must be 0 (float) or 1 (double)");
        if (rowStart[rows] != nnz)
            throw std::invalid_argument("bad end of rowStart");
        File F(path, "wb");
        if (!F.f)
            throw std::runtime_error("failed to open output file " + path);
        const int hdr[4] = {dtype, rows, cols, nnz};
        writeN(F.f, hdr, 4, path);
        writeValues(F.f, dtype, values, (size_t)nnz, path);
        writeN(F.f, col, (size_t)nnz, path);
        writeN(F.f, rowStart, (size_t)rows + 1, path);
    }

    BinVec readBinVec(const std::string & path)
    {
        File F(path, "rb");
        if (!F.f)
            throw std::runtime_error("failed to open input file " + path);
        int hdr[2];
        if (!readN(F.f, hdr, 1) || (hdr[0] != 0 && hdr[0] != 1))
            throw std::runtime_error("failed to read vector: bad dtype");
        if (!readN(F.f, hdr + 1, 1))
            throw std::runtime_error("failed to read vector: couldn't read header");
        if (hdr[1] < 1)
            throw std::runtime_error("failed to read vector: bad size");
        BinVec v;
        v.dtype = hdr[0];
        readValues(F.f, v.dtype, (size_t)hdr[1], v.v, "vector");
        return v;
    }

    void writeBinVec(const std::string & path, int n, const double * values, int dtype)
    {
        if (dtype != 0 && dtype != 1)
            throw std::invalid_argument("dtype must be 0 (float) or 1 (double)");
        File F(path, "wb");
        if (!F.f)
            throw std::runtime_error("failed to open output file " + path);
        const int hdr[2] = {dtype, n};
        writeN(F.f, hdr, 2, path);
        writeValues(F.f, dtype, values, (size_t)n, path);
    }
} // namespace nsf
