// Test-only stand-in for the small part of OpenCV's cv::Mat that the reference's element integrator
// (cpp/libs/Element/src/triangleIntegrator.cpp) and its CSR assembly (cpp/libs/Fem/src/chorinCsr.cpp)
// use, so that those two reference files compile into the reference harness (oracle/_ref) without
// OpenCV.  Nothing in the product includes it.
//
// What it provides: dense, owning, row-major 2-D matrices of one channel, float (CV_32FC1) or int32
// (CV_32SC1); create / setTo / ptr / at; the transpose t(); the matrix product A * B and the scalar
// product A * s (float matrices); += and *=.  Products accumulate each dot product in double and
// round once to float.  OpenCV evaluates `A.t() * B * C * s` as GEMM calls whose rounding of these
// 2x2 .. 6x6 products may differ from that in the last bit of a float; the tests that use the
// harness compare with tolerances far above that (about 1e-6 relative).
#pragma once

// standard headers that OpenCV's umbrella header makes visible to its includers
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <string>
#include <cstring>
#include <stdexcept>
#include <vector>

#define CV_32SC1 4
#define CV_32FC1 5

namespace cv
{
    class Mat
    {
    public:
        int rows = 0;
        int cols = 0;

        Mat() = default;
        Mat(int r, int c, int type) { create(r, c, type); }

        int type() const { return type_; }
        bool empty() const { return rows == 0 || cols == 0; }

        // (Re)allocate to r x c of `type`; the contents are unspecified after a reallocation, as in
        // OpenCV (callers set them).  Same shape and type: the buffer is kept.
        void create(int r, int c, int type)
        {
            if (type != CV_32FC1 && type != CV_32SC1)
                throw std::invalid_argument("cv::Mat stand-in: only CV_32FC1 and CV_32SC1");
            if (r == rows && c == cols && type == type_ && !data_.empty())
                return;
            rows = r;
            cols = c;
            type_ = type;
            data_.assign((size_t)r * (size_t)c, 0u);
        }

        template <typename T>
        T * ptr(int r)
        {
            static_assert(sizeof(T) == 4, "4-byte element types only");
            return reinterpret_cast<T *>(data_.data()) + (size_t)r * cols;
        }

        template <typename T>
        const T * ptr(int r) const
        {
            static_assert(sizeof(T) == 4, "4-byte element types only");
            return reinterpret_cast<const T *>(data_.data()) + (size_t)r * cols;
        }

        template <typename T>
        T & at(int r, int c)
        {
            return ptr<T>(r)[c];
        }

        template <typename T>
        const T & at(int r, int c) const
        {
            return ptr<T>(r)[c];
        }

        Mat & setTo(double v)
        {
            for (int r = 0; r < rows; r++)
                for (int c = 0; c < cols; c++)
                {
                    if (type_ == CV_32FC1)
                        at<float>(r, c) = (float)v;
                    else
                        at<int>(r, c) = (int)v;
                }
            return *this;
        }

        Mat t() const
        {
            Mat o(cols, rows, type_);
            for (int r = 0; r < rows; r++)
                for (int c = 0; c < cols; c++)
                    std::memcpy(&o.data_[(size_t)c * rows + r], &data_[(size_t)r * cols + c], 4);
            return o;
        }

        Mat & operator*=(double s)
        {
            requireFloat();
            for (auto & w : data_)
            {
                float f;
                std::memcpy(&f, &w, 4);
                f = (float)((double)f * s);
                std::memcpy(&w, &f, 4);
            }
            return *this;
        }

        Mat & operator+=(const Mat & o)
        {
            requireFloat();
            if (o.rows != rows || o.cols != cols || o.type_ != type_)
                throw std::invalid_argument("cv::Mat stand-in: += of different shapes");
            for (int r = 0; r < rows; r++)
                for (int c = 0; c < cols; c++)
                    at<float>(r, c) += o.at<float>(r, c);
            return *this;
        }

        void requireFloat() const
        {
            if (type_ != CV_32FC1)
                throw std::invalid_argument("cv::Mat stand-in: arithmetic on float matrices only");
        }

    private:
        int type_ = CV_32FC1;
        std::vector<unsigned> data_;
    };

    inline Mat operator*(const Mat & a, const Mat & b)
    {
        a.requireFloat();
        b.requireFloat();
        if (a.cols != b.rows)
            throw std::invalid_argument("cv::Mat stand-in: product of incompatible shapes");
        Mat o(a.rows, b.cols, CV_32FC1);
        for (int r = 0; r < a.rows; r++)
            for (int c = 0; c < b.cols; c++)
            {
                double s = 0;
                for (int k = 0; k < a.cols; k++)
                    s += (double)a.at<float>(r, k) * (double)b.at<float>(k, c);
                o.at<float>(r, c) = (float)s;
            }
        return o;
    }

    inline Mat operator*(const Mat & a, double s)
    {
        Mat o = a;
        o *= s;
        return o;
    }

    inline Mat operator*(double s, const Mat & a) { return a * s; }
} // namespace cv
