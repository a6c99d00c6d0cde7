/* vla.h -- the one routine of QLL's internal vla.h (include/vla.h:85,
 * lib/vla.c:1635-1665) that this library exports: makeU, the
 * re-unitarisation QLL's test programs (stress.c:156, fieldtest.c:125) use
 * to turn arbitrary matrices into unitary link fields.
 *
 * makeUD/makeUF(mm, nc, i0, i1) replace sites [i0, i1) of mm, each 2 nc^2
 * reals (nc vectors of nc complex numbers, re/im interleaved) in QLL's
 * one-lane site order, by their Gram-Schmidt orthonormalisation in the
 * reference's order: vector i is normalised, then for each earlier vector
 * j its projection is removed and it is normalised again.  It runs on the
 * GPU, one thread a site; nc is at most 3.  As in QLL the call returns
 * nothing; a failure leaves mm untouched and records a message
 * (qllg_last_error in qll_gb300.h).  The reference takes a thread's share
 * [i0, i1) of the sites from its OpenMP loop; here one call may cover all
 * of them. */
#ifndef QLLG_VLA_H
#define QLLG_VLA_H

#ifdef __cplusplus
extern "C" {
#endif

void makeUD(double *mm, int nc, int i0, int i1);
void makeUF(float *mm, int nc, int i0, int i1);

#ifdef __cplusplus
}
#endif

#endif
