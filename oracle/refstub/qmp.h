/*
 * qmp.h -- a single-rank stand-in for the QMP message-passing API, enough
 * to compile the reference library as a second CPU oracle (test
 * infrastructure).  With one rank the reference never exchanges a message:
 * its shift code only declares messages for off-rank neighbours, and its
 * global sum over ranks is the identity.  Every call here therefore does
 * nothing and reports success; the declared handles are NULL.
 */
#ifndef QLL_REF_QMP_STUB_H
#define QLL_REF_QMP_STUB_H
/* the real qmp.h brings in the C library headers, and the reference
 * relies on that (lib/cg.c uses stdout through common.h's printf0) */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

typedef int QMP_status_t;
typedef int QMP_bool_t;
typedef void *QMP_msgmem_t;
typedef void *QMP_msghandle_t;
typedef enum { QMP_THREAD_SINGLE, QMP_THREAD_FUNNELED, QMP_THREAD_SERIALIZED,
               QMP_THREAD_MULTIPLE } QMP_thread_level_t;
typedef enum { QMP_CTS_NOT_READY = 0, QMP_CTS_READY = 1 } QMP_clear_to_send_t;
#define QMP_SUCCESS 0

static inline QMP_status_t QMP_init_msg_passing(int *argc, char ***argv, QMP_thread_level_t req,
                                                QMP_thread_level_t *prv)
{ (void)argc; (void)argv; if(prv) *prv = req; return QMP_SUCCESS; }
static inline void QMP_finalize_msg_passing(void) {}
static inline void QMP_abort(int code) { (void)code; }
static inline const char *QMP_error_string(QMP_status_t s) { (void)s; return "no error"; }
static inline int QMP_get_number_of_nodes(void) { return 1; }
static inline int QMP_get_node_number(void) { return 0; }
static inline QMP_status_t QMP_barrier(void) { return QMP_SUCCESS; }
static inline QMP_status_t QMP_sum_double_array(double *x, int n)
{ (void)x; (void)n; return QMP_SUCCESS; }
static inline QMP_status_t QMP_sum_double(double *x) { (void)x; return QMP_SUCCESS; }
static inline QMP_status_t QMP_sum_int(int *x) { (void)x; return QMP_SUCCESS; }
static inline QMP_msgmem_t QMP_declare_msgmem(const void *buf, size_t n)
{ (void)buf; (void)n; return NULL; }
static inline QMP_msghandle_t QMP_declare_send_to(QMP_msgmem_t m, int rank, int prio)
{ (void)m; (void)rank; (void)prio; return NULL; }
static inline QMP_msghandle_t QMP_declare_receive_from(QMP_msgmem_t m, int rank, int prio)
{ (void)m; (void)rank; (void)prio; return NULL; }
static inline QMP_msghandle_t QMP_declare_send_recv_pairs(QMP_msghandle_t *h, int n)
{ (void)h; (void)n; return NULL; }
static inline QMP_status_t QMP_start(QMP_msghandle_t h) { (void)h; return QMP_SUCCESS; }
static inline QMP_status_t QMP_wait(QMP_msghandle_t h) { (void)h; return QMP_SUCCESS; }
static inline QMP_status_t QMP_clear_to_send(QMP_msghandle_t h, QMP_clear_to_send_t c)
{ (void)h; (void)c; return QMP_SUCCESS; }
static inline void QMP_free_msghandle(QMP_msghandle_t h) { (void)h; }
static inline void QMP_free_msgmem(QMP_msgmem_t m) { (void)m; }
#endif
