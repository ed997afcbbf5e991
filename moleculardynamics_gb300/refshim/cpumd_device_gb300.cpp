// Drop-in replacement of cpu/common/Device.cpp and common/NeighborList.cpp of
// vakuras/moleculardynamics' cpumd: the same C++ functions, with the same
// signatures (cpu/common/Device.h:19-23, common/NeighborList.h:30-31), run
// on the GB300 engine through the C ABI of include/mdgb.h.
//
// Build cpumd with this file instead of those two, with -DEQUI (real =
// double, as cpumd is configured) and link libmdgb.so.  Errors end the
// program with a message, as the reference's TC/CPPSAFE_CALL macros do
// (common/Global.h:116-117).
#include "Device.h"
#include "NeighborList.h"
#include "mdgb.h"

#include <cstdlib>
#include <cstring>
#include <iostream>

static_assert(sizeof(real) == sizeof(double), "build cpumd with -DEQUI (real = double)");
static_assert(sizeof(real4) == 4 * sizeof(double) && sizeof(real3) == 3 * sizeof(double),
              "real4/real3 must be the reference layouts");

static void gb300_check(const char* what) {
  int s = mdgb_last_status();
  if (s != MD_OK) {
    std::cerr << "Error: " << what << " failed on the GPU (md_status " << s << ")" << std::endl;
    exit(EXIT_FAILURE);
  }
}

void predict(real4* r, real3* v, real3* a, real3* b, real3* c, real dt, int nop) {
  mdgb_predict((double*)r, (double*)v, (double*)a, (double*)b, (double*)c, dt, nop);
  gb300_check("predict");
}

void correct(real4* r, real3* v, real3* f, real3* a, real3* b, real3* c, real dt, int nop,
             real nPos, bool& flag, float energyLoss) {
  int fl = 0;
  mdgb_correct((double*)r, (double*)v, (const double*)f, (double*)a, (double*)b, (double*)c,
               dt, nop, nPos, &fl, energyLoss);
  gb300_check("correct");
  flag = fl != 0;
}

void lennardJonesForces(real4* posArray, real3* forceArray, int NumberOfParticles,
                        int nlargestsize, int nlistsize, int* list, real rcutsq) {
  mdgb_lennard_jones_forces((const double*)posArray, (double*)forceArray, NumberOfParticles,
                            nlargestsize, nlistsize, list, rcutsq);
  gb300_check("lennardJonesForces");
}

void manyBodyForces(real4* posArray, real3* forceArray, int NumberOfParticles,
                    int nlargestsize, int nlistsize, int* list, real rcutsq, bool ljexist) {
  mdgb_many_body_forces((const double*)posArray, (double*)forceArray, NumberOfParticles,
                        nlargestsize, nlistsize, list, rcutsq, ljexist ? 1 : 0);
  gb300_check("manyBodyForces");
}

void calculateAccelerations(real4* posArray, real3* accelerationArray, real3* forceArray,
                            int NumberOfParticles) {
  mdgb_calculate_accelerations((const double*)posArray, (double*)accelerationArray,
                               (const double*)forceArray, NumberOfParticles);
  gb300_check("calculateAccelerations");
}

// common/NeighborList.cpp:14; the caller frees the list with delete[]
// (cpu/cpumd/Host.cpp:279-286), so the rows are handed over in new[] memory.
int* buildNeighborList(real4* posArray, listSettings* listsettings, real boxSize, int buckets,
                       int NumberOfParticles) {
  mdgb_list_settings s;
  memset(&s, 0, sizeof(s));
  s.rs = listsettings->rs;
  s.rcut = listsettings->rcut;
  int* rows = mdgb_build_neighbor_list((const double*)posArray, &s, boxSize, buckets,
                                       NumberOfParticles);
  gb300_check("buildNeighborList");
  listsettings->nlistsize = s.nlistsize;
  listsettings->nlargestsize = s.nlargestsize;
  size_t total = (size_t)s.nlistsize * (size_t)NumberOfParticles;
  int* list = new int[total > 0 ? total : 1];
  if (total) memcpy(list, rows, sizeof(int) * total);
  mdgb_free(rows);
  return list;
}

// common/NeighborList.cpp:161-207 computeBucket, for code that calls it
// directly (the GPU build itself keeps cells in its own table and never
// calls it).  Same open-addressing scheme and results: the first hash
// H1 cx + H2 cy + H3 cz, on a collision the second hash H1 cx ^ H2 cy ^ H3 cz
// followed by a linear probe; pop = true looks a cell up (-1 if absent),
// pop = false claims its bucket.  The products keep the reference's C
// integer types: H1 does not fit an int, so H1 * c is a 64-bit product, while
// H2 * c and H3 * c are int products that wrap; the combined value is
// truncated to int before the modulo.
namespace {
long long ref_hash_term(long long h, int c) {
  if (h > 0x7fffffffLL) return h * (long long)c;  // long operand: 64-bit product
  return (long long)(int)((unsigned)h * (unsigned)c);  // int product, wrapped
}
int ref_bucket_mod(long long v, int buckets) {
  int n = (int)(unsigned)(unsigned long long)v;  // int n = <long expression>
  n %= buckets;
  return n < 0 ? n + buckets : n;
}
bool cell_is(const int3& b, int cx, int cy, int cz) {
  return b.x == cx && b.y == cy && b.z == cz;
}
}  // namespace

int computeBucket(int cx, int cy, int cz, int3* bucketlist, int buckets, bool pop) {
  const long long t1 = ref_hash_term(H1, cx), t2 = ref_hash_term(H2, cy),
                  t3 = ref_hash_term(H3, cz);
  int n = ref_bucket_mod(t1 + t2 + t3, buckets);
  if (pop && bucketlist[n].x == -1) return -1;
  if (bucketlist[n].x != -1 && !cell_is(bucketlist[n], cx, cy, cz)) {
    // taken by another cell: second hash, then the next free or matching bucket
    n = ref_bucket_mod(t1 ^ t2 ^ t3, buckets);
    if (pop && bucketlist[n].x == -1) return -1;
    while (bucketlist[n].x != -1 && !cell_is(bucketlist[n], cx, cy, cz)) n = (n + 1) % buckets;
  }
  if (!pop) bucketlist[n] = int3{cx, cy, cz};
  return n;
}
