// Compile check: the cu:: shims instantiated with the reference's own linalg::CsrMatrix<float>
// (cpp/libs/LinAlg/include/linalg/csrMatrix.h), as a reference caller would build them.  Compiled
// with -fsyntax-only by tests/test_shims.py where the reference tree is present.
#include <linalg/csrMatrix.h>

#include "cu_gb300_shims.hpp"

void instantiate(const linalg::CsrMatrix<float> & m)
{
    cu::csrF a(m);
    cu::spmv s(a);
    cu::spmm mm(a, 2);
    auto solver = cu::createSolver("gs", 2, m, 100, 1e-6f, 1);
    cu::saxpy(a.rows, s.b.get(), s.b.get(), 1.0f);
    (void)solver->getLastMse(0);
    (void)mm;
}
