/*
 * Stand-in for the Trilinos TSQR / Teuchos / Kokkos types that the reference's
 * init_tsqr() names (SRC/orth.c:14-46). Test infrastructure only: it lets the
 * reference's SRC/orth.c compile unmodified as a CPU oracle.
 *
 * Trilinos is not vendored with the reference and no version is pinned
 * (make.inc.example:4 links a local ../tpetra/lib), so this stand-in restates the
 * published contract of Tsqr::factorExplicit for one rank: an explicit thin QR of
 * the nrows x ncols panel A, with Q written to Q_local (ldq) and the upper
 * triangular R to R (ldr, strictly lower part zeroed). It uses LAPACK Householder
 * QR (dgeqrf + dorgqr), so the sign of diag(R) follows LAPACK's convention; the
 * reference does not force a sign either (it passes no forceNonnegativeDiagonal).
 */
#ifndef ORACLE_STUB_TSQR_HPP
#define ORACLE_STUB_TSQR_HPP

#include <string>
#include <vector>
#include <mpi.h>

extern "C" {
void scipy_dgeqrf_(int *m, int *n, double *a, int *lda, double *tau, double *work,
                   int *lwork, int *info);
void scipy_dorgqr_(int *m, int *n, int *k, double *a, int *lda, double *tau,
                   double *work, int *lwork, int *info);
}

namespace Teuchos {
template <class T>
class RCP {
  public:
    RCP() : p_(nullptr) {}
    explicit RCP(T *p) : p_(p) {}
    T *get() const { return p_; }
    T *operator->() const { return p_; }
  private:
    T *p_;  // objects live for the process lifetime; the oracle is short-lived
};
template <class T>
RCP<T> rcp(T *p) { return RCP<T>(p); }
template <class To, class From>
RCP<To> rcp_implicit_cast(const RCP<From> &r) { return RCP<To>(static_cast<To *>(r.get())); }

template <class Ordinal>
class MpiComm {
  public:
    explicit MpiComm(MPI_Comm c) : comm_(c) {}
  private:
    MPI_Comm comm_;
};
}  // namespace Teuchos

namespace Kokkos {
struct DefaultExecutionSpace {
    struct device_type {};
};
}  // namespace Kokkos

namespace TSQR {
template <class Scalar>
class MessengerBase {
  public:
    virtual ~MessengerBase() {}
};

template <class Scalar>
class TeuchosMessenger : public MessengerBase<Scalar> {
  public:
    explicit TeuchosMessenger(const Teuchos::RCP<Teuchos::MpiComm<int> > &) {}
};

template <class LO, class Scalar>
class NodeTsqr {};

template <class LO, class Scalar>
class DistTsqr {
  public:
    void init(const Teuchos::RCP<MessengerBase<Scalar> > &) {}
};

template <class Scalar, class LO, class Device>
struct NodeTsqrFactory {
    static Teuchos::RCP<NodeTsqr<LO, Scalar> > getNodeTsqr(const std::string &) {
        return Teuchos::rcp(new NodeTsqr<LO, Scalar>());
    }
};

template <class LO, class Scalar>
class Tsqr {
  public:
    Tsqr(const Teuchos::RCP<NodeTsqr<LO, Scalar> > &, const Teuchos::RCP<DistTsqr<LO, Scalar> > &) {}

    /* Explicit thin QR of A (nrows x ncols, lda). A is overwritten. */
    void factorExplicit(LO nrows, LO ncols, Scalar A[], LO lda, Scalar Q[], LO ldq,
                        Scalar R[], LO ldr, bool /*contiguousCacheBlocks*/) {
        int m = nrows, n = ncols, la = lda, info = 0, lwork = -1;
        if (n <= 0) return;
        std::vector<double> tau((size_t)n);
        double wq = 0.0;
        scipy_dgeqrf_(&m, &n, A, &la, tau.data(), &wq, &lwork, &info);
        int lw1 = (int)wq;
        lwork = -1;
        scipy_dorgqr_(&m, &n, &n, A, &la, tau.data(), &wq, &lwork, &info);
        int lw2 = (int)wq;
        lwork = lw1 > lw2 ? lw1 : lw2;
        if (lwork < n) lwork = n;
        std::vector<double> work((size_t)lwork);
        scipy_dgeqrf_(&m, &n, A, &la, tau.data(), work.data(), &lwork, &info);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
                R[i + (size_t)j * ldr] = (i <= j) ? A[i + (size_t)j * la] : 0.0;
        scipy_dorgqr_(&m, &n, &n, A, &la, tau.data(), work.data(), &lwork, &info);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i)
                Q[i + (size_t)j * ldq] = A[i + (size_t)j * la];
    }
};
}  // namespace TSQR

#endif
