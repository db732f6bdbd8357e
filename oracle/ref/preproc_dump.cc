// preproc_dump.cc -- project-written createfunky for the oracle build of the
// reference's preprocessor (src/preproc/preprocess.cc).  The reference's
// createfunky (createfunky.cc:32) writes funkyNNNN.h5 through HDF5; this one
// appends the same records to funky_dump.bin in the working directory:
//   int32 myid; double htvars[nhtvars]; int64 nbuckets; then per bucket
//   uint32 key[KEYLENGTH]; int32 buckettype, myproc; int32 bucket_index[6];
//   double xcoord[2], ycoord[2], zcoord[2]; uint32 neighs[NEIGH_SIZE*KEYLENGTH];
//   int32 neigh_proc[NEIGH_SIZE]; then int64 npartition; uint32 partition[].
// It also supplies the original domain (ORACLE_DOMAIN, see cfg_preproc.h).
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <vector>
using namespace std;
#include <buckstr.h>

double oracle_pre_Ll[3] = { 0, 0, 0 };
double oracle_pre_Lu[3] = { 1, 1, 1 };

namespace {
struct DomainFromEnv {
  DomainFromEnv() {
    const char *s = getenv("ORACLE_DOMAIN");
    if (!s) return;
    double v[6];
    if (sscanf(s, "%lf %lf %lf %lf %lf %lf", v, v + 1, v + 2, v + 3, v + 4, v + 5) != 6) {
      fprintf(stderr, "ORACLE_DOMAIN: six numbers expected\n");
      exit(2);
    }
    for (int a = 0; a < 3; a++) {
      oracle_pre_Ll[a] = v[a];
      oracle_pre_Lu[a] = v[3 + a];
    }
  }
} domain_from_env;
}  // namespace

void createfunky(int myid, int nhtvars, double *htvars, vector<BucketStruct> &bg, vector<unsigned> &partition) {
  FILE *f = fopen("funky_dump.bin", "ab");
  if (!f) {
    perror("funky_dump.bin");
    exit(2);
  }
  int32_t id = myid;
  fwrite(&id, 4, 1, f);
  fwrite(htvars, sizeof(double), nhtvars, f);
  int64_t nb = (int64_t)bg.size();
  fwrite(&nb, 8, 1, f);
  for (size_t b = 0; b < bg.size(); b++) {
    const BucketStruct &s = bg[b];
    fwrite(s.key, 4, KEYLENGTH, f);
    int32_t t[2] = { s.buckettype, s.myproc };
    fwrite(t, 4, 2, f);
    fwrite(s.bucket_index, 4, 6, f);
    fwrite(s.xcoord, 8, 2, f);
    fwrite(s.ycoord, 8, 2, f);
    fwrite(s.zcoord, 8, 2, f);
    fwrite(s.neighs, 4, NEIGH_SIZE * KEYLENGTH, f);
    fwrite(s.neigh_proc, 4, NEIGH_SIZE, f);
  }
  int64_t np = (int64_t)partition.size();
  fwrite(&np, 8, 1, f);
  if (np) fwrite(partition.data(), 4, np, f);
  fclose(f);
}
