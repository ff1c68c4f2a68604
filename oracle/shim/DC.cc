/* Oracle (test infrastructure only): implementation of the DC-lib stand-in. */
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <vector>
#include <algorithm>

#include "DC.h"

static uint64_t now_ns ()
{
    timespec ts;
    clock_gettime (CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

void DC_timer::start_cycles () { t0 = now_ns (); }
void DC_timer::stop_cycles () { total += now_ns () - t0; count++; }
uint64_t DC_timer::get_avg_cycles () { return count ? total / count : 0; }
void DC_timer::start_time () { s0 = now_ns () * 1e-9; }
void DC_timer::stop_time () { stotal += now_ns () * 1e-9 - s0; scount++; }
double DC_timer::get_avg_time () { return scount ? stotal / scount : 0.0; }
void DC_timer::reset_time () { stotal = 0; scount = 0; }

const char *DC_data_path ()
{
    const char *p = getenv ("MINIFEM_DATA_PATH");
    return p ? p : ".";
}

void DC_create_nodeToElem (index_t &nodeToElem, int *elemToNode, int nbElem,
                           int dimElem, int nbNodes)
{
    int *idx = nodeToElem.index, *val = nodeToElem.value;
    std::vector<int> fill (nbNodes, 0);
    memset (idx, 0, sizeof (int) * (nbNodes + 1));
    for (long i = 0; i < (long)nbElem * dimElem; i++) idx[elemToNode[i]]++;
    for (int i = 0; i < nbNodes; i++) idx[i + 1] += idx[i];
    for (int e = 0; e < nbElem; e++)
        for (int k = 0; k < dimElem; k++) {
            int n = elemToNode[(long)e * dimElem + k] - 1;
            val[idx[n] + fill[n]++] = e;
        }
}

void DC_create_elemToElem (list_t *elemToElem, index_t &nodeToElem, int *elemToNode,
                           int firstElem, int lastElem, int dimElem)
{
    std::vector<int> buf;
    for (int e = firstElem; e <= lastElem; e++) {
        buf.clear ();
        for (int k = 0; k < dimElem; k++) {
            int n = elemToNode[(long)e * dimElem + k] - 1;
            for (int j = nodeToElem.index[n]; j < nodeToElem.index[n + 1]; j++)
                if (nodeToElem.value[j] != e) buf.push_back (nodeToElem.value[j]);
        }
        std::sort (buf.begin (), buf.end ());
        buf.erase (std::unique (buf.begin (), buf.end ()), buf.end ());
        list_t &l = elemToElem[e - firstElem];
        l.size = (int)buf.size ();
        l.list = new int [buf.size () + 1];
        std::copy (buf.begin (), buf.end (), l.list);
    }
}

void DC_create_permutation (int *perm, int *colorPart, int nbItem, int nbColors)
{
    std::vector<int> start (nbColors + 1, 0);
    for (int i = 0; i < nbItem; i++) start[colorPart[i] + 1]++;
    for (int c = 0; c < nbColors; c++) start[c + 1] += start[c];
    for (int i = 0; i < nbItem; i++) perm[i] = start[colorPart[i]]++;
}

void DC_permute_int_2d_array (int *array, int *perm, int nbItem, int dimItem,
                              int offset)
{
    (void)offset;
    std::vector<int> tmp (array, array + (long)nbItem * dimItem);
    for (int i = 0; i < nbItem; i++)
        for (int k = 0; k < dimItem; k++)
            array[(long)perm[i] * dimItem + k] = tmp[(long)i * dimItem + k];
}
