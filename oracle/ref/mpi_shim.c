/*
 * Process-based MPI replacement for running the unmodified PIMD-B++
 * reference as a CPU oracle.  Test infrastructure only.
 *
 * Model: MPI_Init maps one anonymous shared region, then forks
 * PIMDB_SHIM_NP-1 children; rank r is the r-th process.  All collectives are
 * implemented with a process-shared, sense-reversing barrier that gives up
 * after PIMDB_SHIM_TIMEOUT seconds (default 300) so a rank that died never
 * leaves the others blocked forever.
 *
 *  - MPI_Sendrecv: every rank posts its message in its own mailbox slot,
 *    barrier, reads the slot of `source`, barrier.  This matches the only
 *    pattern the reference uses (every rank calls it at the same point, ring
 *    neighbours; src/simulation.cpp:302-346).
 *  - MPI_Allreduce(SUM, double): post, barrier, sum slots in rank order,
 *    barrier (src/simulation.cpp:595, src/observables/observable.cpp:105).
 *  - MPI_Win_allocate_shared: deterministic bump allocation in a shared heap
 *    mapped before the fork, so the addresses agree in every rank
 *    (src/normal_modes.cpp:15-45).
 */
#define _GNU_SOURCE
#include "mpi.h"

#include <errno.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

#define SHIM_MAX_RANKS 1024
#define SHIM_SLOT_BYTES (1u << 20)
#define SHIM_HEAP_BYTES (1ul << 33)
#define SHIM_MAX_WINDOWS 65536

typedef struct {
    pthread_mutex_t mu;
    pthread_cond_t cv;
    int count;
    int generation;
    int nproc;
    int failed;
    long heap_top;
    long win_size[SHIM_MAX_RANKS];
    int slot_dest[SHIM_MAX_RANKS];
    int slot_count[SHIM_MAX_RANKS];
} shim_ctl;

typedef struct {
    long* base; /* [nproc] */
    long* size; /* [nproc] */
} shim_window;

static shim_ctl* g_ctl = NULL;
static unsigned char* g_slots = NULL;
static unsigned char* g_heap = NULL;
static int g_rank = 0;
static int g_nproc = 1;
static pid_t g_children[SHIM_MAX_RANKS];
static shim_window g_windows[SHIM_MAX_WINDOWS];
static int g_nwindows = 0;
static double g_timeout = 300.0;

static void shim_die(const char* what) {
    fprintf(stderr, "[mpi-shim] rank %d: %s\n", g_rank, what);
    fflush(stderr);
    if (g_ctl) g_ctl->failed = 1;
    _exit(3);
}

static void* shim_map(size_t bytes) {
    void* p = mmap(NULL, bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (p == MAP_FAILED) shim_die("mmap failed");
    return p;
}

static void shim_barrier(void) {
    if (g_nproc == 1) return;
    pthread_mutex_lock(&g_ctl->mu);
    int gen = g_ctl->generation;
    if (++g_ctl->count == g_nproc) {
        g_ctl->count = 0;
        g_ctl->generation++;
        pthread_cond_broadcast(&g_ctl->cv);
    } else {
        struct timespec dl;
        clock_gettime(CLOCK_REALTIME, &dl);
        dl.tv_sec += (time_t)g_timeout;
        while (gen == g_ctl->generation && !g_ctl->failed) {
            int rc = pthread_cond_timedwait(&g_ctl->cv, &g_ctl->mu, &dl);
            if (rc == ETIMEDOUT) {
                pthread_mutex_unlock(&g_ctl->mu);
                shim_die("barrier timed out (another rank probably failed)");
            }
        }
        if (g_ctl->failed) {
            pthread_mutex_unlock(&g_ctl->mu);
            shim_die("another rank failed");
        }
    }
    pthread_mutex_unlock(&g_ctl->mu);
}

int MPI_Init(int* argc, char*** argv) {
    (void)argc;
    (void)argv;
    const char* np = getenv("PIMDB_SHIM_NP");
    const char* to = getenv("PIMDB_SHIM_TIMEOUT");
    g_nproc = np ? atoi(np) : 1;
    if (g_nproc < 1 || g_nproc > SHIM_MAX_RANKS) shim_die("PIMDB_SHIM_NP out of range");
    if (to) g_timeout = atof(to);

    g_ctl = (shim_ctl*)shim_map(sizeof(shim_ctl));
    g_slots = (unsigned char*)shim_map((size_t)SHIM_SLOT_BYTES * (size_t)g_nproc);
    g_heap = (unsigned char*)shim_map(SHIM_HEAP_BYTES);

    pthread_mutexattr_t ma;
    pthread_condattr_t ca;
    pthread_mutexattr_init(&ma);
    pthread_mutexattr_setpshared(&ma, PTHREAD_PROCESS_SHARED);
    pthread_condattr_init(&ca);
    pthread_condattr_setpshared(&ca, PTHREAD_PROCESS_SHARED);
    pthread_mutex_init(&g_ctl->mu, &ma);
    pthread_cond_init(&g_ctl->cv, &ca);
    g_ctl->nproc = g_nproc;

    fflush(NULL);
    for (int r = 1; r < g_nproc; ++r) {
        pid_t pid = fork();
        if (pid < 0) shim_die("fork failed");
        if (pid == 0) {
            g_rank = r;
            return MPI_SUCCESS;
        }
        g_children[r] = pid;
    }
    g_rank = 0;
    return MPI_SUCCESS;
}

int MPI_Finalize(void) {
    shim_barrier();
    if (g_rank == 0) {
        int failed = 0;
        for (int r = 1; r < g_nproc; ++r) {
            int st = 0;
            waitpid(g_children[r], &st, 0);
            if (!WIFEXITED(st) || WEXITSTATUS(st) != 0) failed = 1;
        }
        if (failed || g_ctl->failed) {
            fprintf(stderr, "[mpi-shim] a rank failed\n");
            fflush(NULL);
            _exit(3);
        }
    }
    fflush(NULL);
    return MPI_SUCCESS;
}

int MPI_Comm_rank(MPI_Comm comm, int* rank) {
    (void)comm;
    *rank = g_rank;
    return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int* size) {
    (void)comm;
    *size = g_nproc;
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm comm) {
    (void)comm;
    shim_barrier();
    return MPI_SUCCESS;
}

double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status) {
    (void)sendtype;
    (void)sendtag;
    (void)recvtype;
    (void)recvtag;
    (void)comm;
    (void)status;
    size_t sbytes = (size_t)sendcount * sizeof(double);
    size_t rbytes = (size_t)recvcount * sizeof(double);
    if (sbytes > SHIM_SLOT_BYTES || rbytes > SHIM_SLOT_BYTES) shim_die("message larger than a mailbox slot");
    if (g_nproc == 1) {
        memmove(recvbuf, sendbuf, rbytes < sbytes ? rbytes : sbytes);
        return MPI_SUCCESS;
    }
    memcpy(g_slots + (size_t)g_rank * SHIM_SLOT_BYTES, sendbuf, sbytes);
    g_ctl->slot_dest[g_rank] = dest;
    g_ctl->slot_count[g_rank] = sendcount;
    shim_barrier();
    if (g_ctl->slot_dest[source] != g_rank || g_ctl->slot_count[source] != recvcount)
        shim_die("Sendrecv pattern is not a matched exchange");
    memcpy(recvbuf, g_slots + (size_t)source * SHIM_SLOT_BYTES, rbytes);
    shim_barrier();
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
                  MPI_Comm comm) {
    (void)datatype;
    (void)op;
    (void)comm;
    size_t bytes = (size_t)count * sizeof(double);
    if (bytes > SHIM_SLOT_BYTES) shim_die("Allreduce buffer larger than a mailbox slot");
    if (g_nproc == 1) {
        memmove(recvbuf, sendbuf, bytes);
        return MPI_SUCCESS;
    }
    memcpy(g_slots + (size_t)g_rank * SHIM_SLOT_BYTES, sendbuf, bytes);
    shim_barrier();
    double* out = (double*)recvbuf;
    for (int i = 0; i < count; ++i) {
        double s = 0.0;
        for (int r = 0; r < g_nproc; ++r) s += ((const double*)(g_slots + (size_t)r * SHIM_SLOT_BYTES))[i];
        out[i] = s;
    }
    shim_barrier();
    return MPI_SUCCESS;
}

int MPI_Win_allocate_shared(MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm, void* baseptr,
                            MPI_Win* win) {
    (void)disp_unit;
    (void)info;
    (void)comm;
    if (g_nwindows >= SHIM_MAX_WINDOWS) shim_die("too many shared windows");
    g_ctl->win_size[g_rank] = size;
    shim_barrier();
    shim_window* w = &g_windows[g_nwindows];
    w->base = (long*)malloc(sizeof(long) * (size_t)g_nproc);
    w->size = (long*)malloc(sizeof(long) * (size_t)g_nproc);
    if (!w->base || !w->size) shim_die("out of memory");
    long top = g_ctl->heap_top;
    for (int r = 0; r < g_nproc; ++r) {
        long sz = g_ctl->win_size[r];
        w->base[r] = top;
        w->size[r] = sz;
        top += (sz + 255) & ~255L;
    }
    if (top > (long)SHIM_HEAP_BYTES) shim_die("shared heap exhausted");
    shim_barrier();
    if (g_rank == 0) g_ctl->heap_top = top;
    shim_barrier();
    *(void**)baseptr = w->size[g_rank] > 0 ? (void*)(g_heap + w->base[g_rank]) : NULL;
    *win = g_nwindows++;
    return MPI_SUCCESS;
}

int MPI_Win_shared_query(MPI_Win win, int rank, MPI_Aint* size, int* disp_unit, void* baseptr) {
    if (win < 0 || win >= g_nwindows || rank < 0 || rank >= g_nproc) shim_die("bad window query");
    shim_window* w = &g_windows[win];
    *size = w->size[rank];
    *disp_unit = (int)sizeof(double);
    *(void**)baseptr = w->size[rank] > 0 ? (void*)(g_heap + w->base[rank]) : NULL;
    return MPI_SUCCESS;
}

int MPI_Win_free(MPI_Win* win) {
    (void)win;
    shim_barrier();
    return MPI_SUCCESS;
}
