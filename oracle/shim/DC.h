/* Oracle (test infrastructure only): stand-in for the external DC-lib header.
 *
 * The reference includes <DC.h> (src/main.cc:26, src/headers/FEM.h:23,
 * src/headers/assembly.h:20, src/headers/matrix.h:20, src/headers/coloring.h:20,
 * src/headers/halo.h:23) from DC-lib, which is not vendored.  This header gives
 * only what the REF and COLORING builds use: the timer, the index/list types,
 * MAX_ELEM_PER_PART and four mesh helpers, written from how the reference calls
 * them (src/main.cc:117,229,243-247; src/coloring.cc:90-107).  The timer reports
 * nanoseconds where DC-lib reported RDTSC cycles.
 */
#ifndef ORACLE_SHIM_DC_H
#define ORACLE_SHIM_DC_H

#include <cstdint>
#include <string>

#define MAX_ELEM_PER_PART 0

typedef struct index_s {
    int *index = nullptr;
    int *value = nullptr;
} index_t;

typedef struct list_s {
    int *list = nullptr;
    int size = 0;
    ~list_s () { delete[] list; }
} list_t;

class DC_timer {
public:
    void start_cycles ();
    void stop_cycles ();
    uint64_t get_avg_cycles ();
    void start_time ();
    void stop_time ();
    double get_avg_time ();
    void reset_time ();
private:
    uint64_t t0 = 0, total = 0, count = 0;
    double s0 = 0, stotal = 0;
    uint64_t scount = 0;
};

/* Root of the mesh data tree: $MINIFEM_DATA_PATH, default "." */
const char *DC_data_path ();

/* Node -> element lists, ascending element id per node; element ids 0-based. */
void DC_create_nodeToElem (index_t &nodeToElem, int *elemToNode, int nbElem,
                           int dimElem, int nbNodes);

/* For each element of [firstElem, lastElem]: the other elements sharing a node. */
void DC_create_elemToElem (list_t *elemToElem, index_t &nodeToElem, int *elemToNode,
                           int firstElem, int lastElem, int dimElem);

/* perm[old] = new position; stable counting sort of items by colour. */
void DC_create_permutation (int *perm, int *colorPart, int nbItem, int nbColors);

/* array'[perm[i]] = array[i] for rows of dimItem ints. */
void DC_permute_int_2d_array (int *array, int *perm, int nbItem, int dimItem,
                              int offset);

#endif
