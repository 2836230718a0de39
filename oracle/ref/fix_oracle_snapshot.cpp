/* Test infrastructure only (see fix_oracle_snapshot.h).  Dumps the reference's
 * own in-memory state so the CPU restatement and the GPU path can be compared
 * against it bit for bit (pair sets) or within tolerance (forces).
 *
 * File layout (all little-endian, SoA):
 *   char[8] "DEMSNAP1"; int64 step;
 *   int32 nlocal, nghost, dnum, nwallhist;
 *   double boxlo[3], boxhi[3]; int32 periodic[3], pad;
 *   int32 tag[nall], type[nall];
 *   double x[3*nall], v[3*nall], omega[3*nall], f[3*nall], torque[3*nall],
 *          radius[nall], rmass[nall];
 *   int32 npairs; int32 i[npairs], j[npairs], flag[npairs];
 *   double hist[npairs*dnum];
 *   nwallhist times: int32 namelen; char name[namelen]; int32 wdnum;
 *                    double data[nlocal*wdnum]
 * Pair (i, j) are local/ghost indices into the atom arrays above, in the
 * order of the reference's granular half list (src/neigh_gran.cpp:485-644).
 */
#include "fix_oracle_snapshot.h"
#include "atom.h"
#include "comm.h"
#include "domain.h"
#include "error.h"
#include "force.h"
#include "modify.h"
#include "neigh_list.h"
#include "pair_gran.h"
#include "update.h"
#include "fix_property_atom.h"
#include "fix_mesh_surface.h"
#include "fix_contact_history_mesh.h"
#include "tri_mesh.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdint.h>

using namespace LAMMPS_NS;
using namespace FixConst;

FixOracleSnapshot::FixOracleSnapshot(LAMMPS *lmp, int narg, char **arg) :
  Fix(lmp, narg, arg)
{
  if (narg < 5) error->all(FLERR,"Illegal fix oracle/snapshot command");
  prefix_ = arg[3];
  for (int k = 4; k < narg; k++) steps_.push_back(atol(arg[k]));
  nevery = 1;
}

int FixOracleSnapshot::setmask()
{
  return END_OF_STEP;
}

void FixOracleSnapshot::setup(int)
{
  for (size_t k = 0; k < steps_.size(); k++)
    if (steps_[k] == update->ntimestep) { write_snapshot(); return; }
}

void FixOracleSnapshot::end_of_step()
{
  for (size_t k = 0; k < steps_.size(); k++)
    if (steps_[k] == update->ntimestep) { write_snapshot(); return; }
}

template <typename T>
static void put(FILE *fp, const T *p, size_t n) { fwrite(p, sizeof(T), n, fp); }

void FixOracleSnapshot::write_snapshot()
{
  char fname[1024];
  snprintf(fname, sizeof(fname), "%s.%ld.bin", prefix_.c_str(), (long)update->ntimestep);
  FILE *fp = fopen(fname, "wb");
  if (!fp) error->one(FLERR,"oracle/snapshot: cannot open output file");

  const int nlocal = atom->nlocal, nghost = atom->nghost, nall = nlocal + nghost;
  PairGran *pg = dynamic_cast<PairGran*>(force->pair);
  const int dnum = pg ? pg->dnum() : 0;

  std::vector<int> wall_idx;
  for (int k = 0; k < modify->nfix; k++)
    if (strncmp(modify->fix[k]->id, "history_", 8) == 0 &&
        strcmp(modify->fix[k]->style, "property/atom") == 0)
      wall_idx.push_back(k);

  fwrite("DEMSNAP1", 1, 8, fp);
  int64_t step = update->ntimestep;
  put(fp, &step, 1);
  int32_t hdr[4] = {nlocal, nghost, dnum, (int32_t)wall_idx.size()};
  put(fp, hdr, 4);
  put(fp, domain->boxlo, 3);
  put(fp, domain->boxhi, 3);
  int32_t per[4] = {domain->xperiodic, domain->yperiodic, domain->zperiodic, 0};
  put(fp, per, 4);

  std::vector<int32_t> ibuf(nall);
  for (int i = 0; i < nall; i++) ibuf[i] = atom->tag[i];
  put(fp, ibuf.data(), nall);
  for (int i = 0; i < nall; i++) ibuf[i] = atom->type[i];
  put(fp, ibuf.data(), nall);
  double **vec3[5] = {atom->x, atom->v, atom->omega, atom->f, atom->torque};
  std::vector<double> dbuf(3 * (size_t)nall);
  for (int a = 0; a < 5; a++) {
    for (int i = 0; i < nall; i++)
      for (int d = 0; d < 3; d++) dbuf[3 * (size_t)i + d] = vec3[a][i][d];
    put(fp, dbuf.data(), 3 * (size_t)nall);
  }
  put(fp, atom->radius, nall);
  put(fp, atom->rmass, nall);

  std::vector<int32_t> pi, pj, pf;
  std::vector<double> ph;
  if (pg && pg->list) {
    NeighList *list = pg->list;
    NeighList *hl = pg->listgranhistory;
    for (int ii = 0; ii < list->inum; ii++) {
      const int i = list->ilist[ii];
      for (int jj = 0; jj < list->numneigh[i]; jj++) {
        pi.push_back(i);
        pj.push_back(list->firstneigh[i][jj] & NEIGHMASK);
        pf.push_back(hl ? hl->firstneigh[i][jj] : 0);
        for (int d = 0; d < dnum; d++)
          ph.push_back(hl ? hl->firstdouble[i][dnum * jj + d] : 0.0);
      }
    }
  }
  int32_t np = (int32_t)pi.size();
  put(fp, &np, 1);
  put(fp, pi.data(), np);
  put(fp, pj.data(), np);
  put(fp, pf.data(), np);
  put(fp, ph.data(), ph.size());

  for (size_t k = 0; k < wall_idx.size(); k++) {
    FixPropertyAtom *fpa = static_cast<FixPropertyAtom*>(modify->fix[wall_idx[k]]);
    const char *name = fpa->id;
    int32_t len = (int32_t)strlen(name);
    put(fp, &len, 1);
    fwrite(name, 1, len, fp);
    int32_t wd = fpa->get_nvalues();
    put(fp, &wd, 1);
    std::vector<double> w((size_t)nlocal * wd);
    for (int i = 0; i < nlocal; i++)
      for (int d = 0; d < wd; d++)
        w[(size_t)i * wd + d] = (wd == 1 && fpa->vector_atom) ? fpa->vector_atom[i]
                                                              : fpa->array_atom[i][d];
    put(fp, w.data(), w.size());
  }

  // triangle meshes of fix mesh/surface: geometry, edge/corner activity
  // (SurfaceMesh::buildNeighbours) and the per-atom mesh contact slots of
  // FixContactHistoryMesh (partner triangle id or -1, history)
  std::vector<FixMeshSurface*> meshes;
  for (int k = 0; k < modify->nfix; k++)
    if (strcmp(modify->fix[k]->style, "mesh/surface") == 0)
      meshes.push_back(static_cast<FixMeshSurface*>(modify->fix[k]));
  int32_t nm = (int32_t)meshes.size();
  put(fp, &nm, 1);
  for (size_t k = 0; k < meshes.size(); k++) {
    FixMeshSurface *fm = meshes[k];
    TriMesh *mesh = fm->triMesh();
    int32_t len = (int32_t)strlen(fm->id);
    put(fp, &len, 1);
    fwrite(fm->id, 1, len, fp);
    int32_t ntri = mesh->sizeLocal();
    put(fp, &ntri, 1);
    std::vector<int32_t> ids(ntri);
    std::vector<double> nodes(9 * (size_t)ntri);
    std::vector<uint8_t> act(6 * (size_t)ntri);
    for (int t = 0; t < ntri; t++) {
      ids[t] = mesh->id(t);
      for (int q = 0; q < 3; q++) {
        mesh->node(t, q, &nodes[9 * (size_t)t + 3 * q]);
        act[6 * (size_t)t + q] = mesh->edgeActive(t, q) ? 1 : 0;
        act[6 * (size_t)t + 3 + q] = mesh->cornerActive(t, q) ? 1 : 0;
      }
    }
    put(fp, ids.data(), ntri);
    put(fp, nodes.data(), nodes.size());
    put(fp, act.data(), act.size());
    FixContactHistoryMesh *ch = fm->contactHistory();
    int32_t md = ch ? ch->get_dnum() : 0;
    put(fp, &md, 1);
    std::vector<int32_t> nslot(nlocal, 0), npart(nlocal, 0), part;
    std::vector<double> mh;
    if (ch) {
      for (int i = 0; i < nlocal; i++) {
        nslot[i] = ch->nneighs(i);
        npart[i] = ch->n_partner(i);
        for (int s = 0; s < nslot[i]; s++) {
          part.push_back(ch->get_partner_idTri(i, s));
          const double *h = ch->contacthistory(i, s);
          for (int d = 0; d < md; d++) mh.push_back(h[d]);
        }
      }
    }
    put(fp, nslot.data(), nlocal);
    put(fp, npart.data(), nlocal);
    int32_t ns = (int32_t)part.size();
    put(fp, &ns, 1);
    put(fp, part.data(), part.size());
    put(fp, mh.data(), mh.size());
  }
  fclose(fp);
}
