/*
 * layout.h -- lattice layout types and functions of QLL's C API (drop-in
 * for the reference's include/layout.h:1-141).
 *
 * The structs keep the reference's member order and types, because callers
 * allocate them themselves (embedqop.c:35-37 puts a StaggeredSolver on the
 * stack) and read members such as Layout.nSites.  This library always sets
 * up the one-rank, one-lane layout (innerGeom = 1, the reference built with
 * -DC1): field index i of a host array [nSites][nelem] is the site numbered
 * by layoutIndex -- even sites first, each parity in lexicographic order
 * with x0 fastest.  The QMP message handles of ShiftIndices/ShiftBuf are
 * pointers in QMP; here they are plain pointers and always NULL.
 */
#ifndef QLLG_LAYOUT_H
#define QLLG_LAYOUT_H

typedef void *qllg_msg_handle;   /* stands for QMP_msgmem_t / QMP_msghandle_t */

typedef struct llist {
  void *value;
  struct llist *next;
} llist;

/* include/layout.h:10-31 */
typedef struct {
  int nDim;
  int *physGeom;
  int *rankGeom;
  int *innerGeom;
  int *outerGeom;
  int *localGeom;
  int physVol;
  int nEven;
  int nOdd;
  int nSites;
  int nEvenOuter;
  int nOddOuter;
  int nSitesOuter;
  int nSitesInner;
  int innerCb;
  int innerCbDir;
  llist *shifts;
  int nranks;
  int myrank;
} Layout;

/* include/layout.h:33-36 */
typedef struct {
  int rank;
  int index;
} LayoutIndex;

/* include/layout.h:38-43 */
typedef struct {
  int begin;
  int end;
  int beginOuter;
  int endOuter;
} Subset;

/* include/layout.h:45-49 */
void layoutSetup(Layout *l);
void layoutIndex(Layout *l, LayoutIndex *li, int coords[]);
void layoutCoord(Layout *l, int coords[], LayoutIndex *li);
void layoutShift(Layout *l, LayoutIndex *li, LayoutIndex *li2, int disp[]);
void layoutSubset(Subset *s, Layout *l, char *sub);

/* include/layout.h:51-61 */
typedef struct {
  int myRank;
  int nIndices;
  int *srcRanks;
  int *srcIndices;
  int nRecvDests;
  int nSendIndices;
  int *sendSrcIndices;
  int *sendDestRanks;
  int *sendDestIndices;
} GatherDescription;

/* include/layout.h:63-84 */
typedef struct {
  GatherDescription *gd;
  int myRank;
  int nIndices;
  int *srcIndices;
  int nRecvRanks;
  int *recvRanks;
  int *recvRankSizes;
  int *recvRankOffsets;
  int recvSize;
  int nRecvDests;
  int *recvDestIndices;
  int *recvBufIndices;
  int nSendRanks;
  int *sendRanks;
  int *sendRankSizes;
  int *sendRankOffsets;
  int sendSize;
  int nSendIndices;
  int *sendIndices;
} GatherIndices;

/* include/layout.h:92-133; only disp, pidx, sidx, vv and perm are filled
 * (one rank: no sends, no receives) */
typedef struct {
  GatherIndices *gi;
  int *disp;
  int *sidx;
  int *pidx;
  int nRecvRanks;
  int *recvRanks;
  int *recvRankSizes;
  int *recvRankSizes1;
  int *recvRankOffsets;
  int *recvRankOffsets1;
  int nRecvSites;
  int nRecvSites1;
  int nRecvDests;
  int *recvDests;
  int *recvLocalSrcs;
  int *recvRemoteSrcs;
  int nSendRanks;
  int *sendRanks;
  int *sendRankSizes;
  int *sendRankSizes1;
  int *sendRankOffsets;
  int *sendRankOffsets1;
  int nSendSites;
  int nSendSites1;
  int *sendSites;
  int vv;
  int offr, lenr, nthreads;
  int perm;
  int pack;
  int blend;
  qllg_msg_handle sqmpmem;
  qllg_msg_handle smsg;
  qllg_msg_handle rqmpmem;
  qllg_msg_handle rmsg;
  qllg_msg_handle pairmsg;
} ShiftIndices;

/* include/layout.h:135-141 */
typedef struct {
  qllg_msg_handle sqmpmem;
  qllg_msg_handle smsg;
  qllg_msg_handle rqmpmem;
  qllg_msg_handle rmsg;
  qllg_msg_handle pairmsg;
  void *sbuf;
  void *rbuf;
  int sbufSize;
  int rbufSize;
  int first;
  int *offr;
  int *lenr;
} ShiftBuf;

#endif
