/* run_style verlet/gb300: see verlet_gb300.h. */

#include "verlet_gb300.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "atom.h"
#include "atom_vec.h"
#include "comm.h"
#include "domain.h"
#include "error.h"
#include "fix.h"
#include "fix_contact_history.h"
#include "fix_gravity_gb300.h"
#include "fix_insert.h"
#include "fix_particledistribution_discrete.h"
#include "fix_mesh_surface.h"
#include "fix_move_mesh_gb300.h"
#include "fix_nve_sphere_gb300.h"
#include "fix_wall_gran_gb300.h"
#include "force.h"
#include "modify.h"
#include "neighbor.h"
#include "output.h"
#include "pair_gran_gb300.h"
#include "timer.h"
#include "tri_mesh.h"
#include "update.h"

using namespace LAMMPS_NS;
using namespace FixConst;

/* run_style verlet/gb300 [capacity N]: N atoms of device room for insertion
   fixes (default: twice the atoms at the first run, at least 10,000 more) */
VerletGB300::VerletGB300(LAMMPS *lmp, int narg, char **arg)
    : Verlet(lmp, narg, arg), h_(NULL), pair_(NULL), capacity_(0), gravity_(NULL), nve_(NULL), natoms_(-1),
      stamp_(0) {
  for (int k = 1; k + 1 < narg; k++)
    if (strcmp(arg[k], "capacity") == 0) capacity_ = atoi(arg[k + 1]);
}

VerletGB300::~VerletGB300() {
  if (h_) dem_destroy(h_);
}

void VerletGB300::check(int rc, const char *what) {
  if (rc == DEM_OK) return;
  char msg[512];
  snprintf(msg, sizeof msg, "verlet/gb300: %s failed (status %d): %s", what, rc, h_ ? dem_last_error(h_) : "");
  error->all(FLERR, msg);
}

/* the styles the device path replaces; every other fix must not run on the
   host between output steps */
void VerletGB300::collect_styles() {
  pair_ = dynamic_cast<PairGranGB300 *>(force->pair);
  if (!pair_) error->all(FLERR, "run_style verlet/gb300 needs pair_style gran/gb300 (run with -sf gb300)");
  walls_.clear();
  movers_.clear();
  inserts_.clear();
  gravity_ = NULL;
  nve_ = NULL;
  int nve = 0;
  const int per_step = INITIAL_INTEGRATE | POST_INTEGRATE | PRE_EXCHANGE | PRE_NEIGHBOR | PRE_FORCE |
                       POST_FORCE | FINAL_INTEGRATE | END_OF_STEP | PRE_INITIAL_INTEGRATE |
                       PRE_FINAL_INTEGRATE;
  // data-only or mesh-maintenance fixes whose host work the device replaces
  static const char *passive[] = {"mesh/surface", "contacthistory", "neighlist/mesh", "property/atom",
                                  "property/global", "multicontact/halfspace"};
  for (int i = 0; i < modify->nfix; i++) {
    Fix *f = modify->fix[i];
    if (FixWallGranGB300 *w = dynamic_cast<FixWallGranGB300 *>(f)) {
      walls_.push_back(w);
      continue;
    }
    if (FixNVESphereGB300 *nv = dynamic_cast<FixNVESphereGB300 *>(f)) {
      nve_ = nv;
      nve++;
      continue;
    }
    if (FixGravityGB300 *g = dynamic_cast<FixGravityGB300 *>(f)) {
      if (gravity_) error->all(FLERR, "verlet/gb300: at most one fix gravity/gb300");
      gravity_ = g;
      continue;
    }
    if (FixMoveMeshGB300 *m = dynamic_cast<FixMoveMeshGB300 *>(f)) {
      movers_.push_back(m);
      continue;
    }
    if (FixInsert *fi = dynamic_cast<FixInsert *>(f)) {  // insert/pack, insert/stream, ...
      inserts_.push_back(fi);
      continue;
    }
    bool skip = false;
    for (size_t k = 0; k < sizeof(passive) / sizeof(passive[0]); k++)
      if (strncmp(f->style, passive[k], strlen(passive[k])) == 0) skip = true;
    if (skip) continue;
    if (modify->fmask[i] & per_step) {
      char msg[512];
      snprintf(msg, sizeof msg,
               "verlet/gb300: fix %s (style %s) runs on the host every step, which the device-resident "
               "loop does not do", f->id, f->style);
      error->all(FLERR, msg);
    }
  }
  if (nve != 1) error->all(FLERR, "verlet/gb300 needs exactly one fix nve/sphere/gb300");
}

void VerletGB300::init() {
  Verlet::init();
  if (comm->nprocs != 1) error->all(FLERR, "verlet/gb300 runs on one MPI rank (one GPU)");
  if (domain->triclinic) error->all(FLERR, "verlet/gb300 needs an orthogonal box");
  if (!atom->map_style) error->all(FLERR, "verlet/gb300 needs an atom map (atom_modify map array)");
  if (!atom->radius_flag || !atom->rmass_flag || !atom->omega_flag || !atom->torque_flag)
    error->all(FLERR, "verlet/gb300 needs atom_style granular");
  collect_styles();
}

/* order-independent 64-bit digest of the host state of the local atoms */
uint64_t VerletGB300::host_stamp() const {
  uint64_t sum = 0;
  for (int i = 0; i < atom->nlocal; i++) {
    uint64_t hsh = 1469598103934665603ULL;
    const unsigned char *parts[] = {(const unsigned char *)atom->x[i], (const unsigned char *)atom->v[i],
                                    (const unsigned char *)atom->omega[i], (const unsigned char *)&atom->radius[i],
                                    (const unsigned char *)&atom->rmass[i], (const unsigned char *)&atom->type[i],
                                    (const unsigned char *)&atom->tag[i]};
    const size_t len[] = {24, 24, 24, 8, 8, sizeof(int), sizeof(int)};
    for (int p = 0; p < 7; p++)
      for (size_t b = 0; b < len[p]; b++) hsh = (hsh ^ parts[p][b]) * 1099511628211ULL;
    sum += hsh;
  }
  return sum;
}

void VerletGB300::create_device() {
  if (h_) dem_destroy(h_);
  h_ = NULL;
  dem_config cfg;
  memset(&cfg, 0, sizeof cfg);
  for (int d = 0; d < 3; d++) {
    cfg.boxlo[d] = domain->boxlo[d];
    cfg.boxhi[d] = domain->boxhi[d];
    cfg.periodic[d] = domain->periodicity[d];
  }
  cfg.dt = update->dt;
  cfg.skin = neighbor->skin;
  cfg.contact_distance_factor = neighbor->contactDistanceFactor;
  cfg.neigh_every = neighbor->every;
  cfg.neigh_delay = neighbor->delay;
  cfg.neigh_check = neighbor->dist_check;
  pair_->fill_config(cfg);
  if (gravity_) {
    cfg.gravity_on = 1;
    gravity_->acceleration(cfg.gravity);
  }
  check(dem_create(&cfg, &h_), "dem_create");
  if (!inserts_.empty()) {
    // room and radius range for the insertion templates (PairGran::init_one
    // sizes the cutoff for them the same way)
    double rmin = 0.0, rmax = 0.0;
    for (size_t k = 0; k < inserts_.size(); k++) {
      FixParticledistributionDiscrete *dist = inserts_[k]->get_distribution();
      rmax = std::max(rmax, inserts_[k]->max_r_bound());
      if (!dist) continue;
      for (int t = inserts_[k]->min_type(); t <= inserts_[k]->max_type(); t++) {
        const double r = dist->min_rad(t);
        if (r > 0.0 && r < 1000.0) rmin = rmin > 0.0 ? std::min(rmin, r) : r;
      }
    }
    const long cap = capacity_ > 0 ? capacity_ : std::max<long>(2 * atom->natoms, atom->natoms + 10000);
    check(dem_set_capacity(h_, (int)cap, rmin, rmax), "dem_set_capacity");
  }
  pair_->upload_params(h_);
  for (size_t w = 0; w < walls_.size(); w++) walls_[w]->upload(h_, atom->ntypes);
  for (size_t k = 0; k < movers_.size(); k++) {
    bool found = false;
    for (size_t w = 0; w < walls_.size(); w++)
      for (size_t m = 0; m < walls_[w]->mesh_ids().size(); m++)
        if (walls_[w]->mesh_ids()[m] == movers_[k]->mesh_id()) {
          if (movers_[k]->rotating())
            check(dem_set_mesh_rotation(h_, walls_[w]->device_mesh_ids()[m], movers_[k]->origin(),
                                        movers_[k]->axis(), movers_[k]->period()),
                  "dem_set_mesh_rotation");
          else
            check(dem_set_mesh_motion(h_, walls_[w]->device_mesh_ids()[m], movers_[k]->velocity()),
                  "dem_set_mesh_motion");
          found = true;
        }
    if (!found) error->all(FLERR, "verlet/gb300: move/mesh/gb300 names a mesh no wall/gran/gb300 uses");
  }

  // atoms in host order
  const int n = atom->nlocal;
  std::vector<int> tag(n), type(n);
  std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), w(3 * (size_t)n), r(n), m(n);
  for (int i = 0; i < n; i++) {
    tag[i] = atom->tag[i];
    type[i] = atom->type[i];
    r[i] = atom->radius[i];
    m[i] = atom->rmass[i];
    for (int d = 0; d < 3; d++) {
      x[3 * i + d] = atom->x[i][d];
      v[3 * i + d] = atom->v[i][d];
      w[3 * i + d] = atom->omega[i][d];
    }
  }
  check(dem_upload_atoms(h_, n, &tag[0], &type[0], &x[0], &v[0], &w[0], &r[0], &m[0]), "dem_upload_atoms");

  // contact history the host holds (read_restart, or a run under the
  // reference's own loop): one entry per (owner, partner) side
  FixContactHistory *fh = pair_->get_fix_history();
  if (fh) {
    int npd = 0, dnum = 0;
    check(dem_npairs(h_, &npd, &dnum), "dem_npairs");
    std::vector<int> own, par;
    std::vector<double> hist;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < fh->n_partner(i); j++) {
        if (fh->get_dnum() != dnum) error->all(FLERR, "verlet/gb300: contact history size differs from the model's");
        own.push_back(atom->tag[i]);
        par.push_back(fh->partner(i, j));
        const double *hv = fh->contacthistory(i, j);
        hist.insert(hist.end(), hv, hv + dnum);
      }
    if (!own.empty())
      check(dem_upload_contact_history(h_, (int)own.size(), &own[0], &par[0], &hist[0]),
            "dem_upload_contact_history");
  }
  for (size_t k = 0; k < walls_.size(); k++) {
    if (!walls_[k]->is_primitive()) continue;
    std::vector<double> wh(3 * (size_t)n, 0.0);
    bool any = false;
    for (int i = 0; i < n; i++) any |= walls_[k]->primitive_history(i, &wh[3 * (size_t)i]);
    if (any) check(dem_upload_wall_history(h_, walls_[k]->device_wall_id(), &wh[0]), "dem_upload_wall_history");
  }
  natoms_ = atom->natoms;
  if (comm->me == 0) {
    char msg[256];
    snprintf(msg, sizeof msg, "verlet/gb300: %d atoms, %d walls resident on the GPU\n", n, (int)walls_.size());
    if (screen) fputs(msg, screen);
    if (logfile) fputs(msg, logfile);
  }
}

/* the device state into the host's local atoms; host atoms the device no
   longer holds (lost through a non-periodic boundary) are deleted */
void VerletGB300::download() {
  int n = 0;
  check(dem_natoms(h_, &n), "dem_natoms");
  tag_.resize(n);
  type_.resize(n);
  r_.resize(n);
  m_.resize(n);
  x_.resize(3 * (size_t)n);
  v_.resize(3 * (size_t)n);
  w_.resize(3 * (size_t)n);
  f_.resize(3 * (size_t)n);
  t_.resize(3 * (size_t)n);
  if (n > 0)
    check(dem_download_atoms(h_, &tag_[0], &type_[0], &x_[0], &v_[0], &w_[0], &f_[0], &t_[0], &r_[0], &m_[0]),
          "dem_download_atoms");
  int nlocal = atom->nlocal;
  std::vector<char> present(nlocal, 0);
  int maxtag = 0;
  for (int k = 0; k < n; k++) maxtag = tag_[k] > maxtag ? tag_[k] : maxtag;
  row_of_tag_.assign(maxtag + 1, -1);
  for (int k = 0; k < n; k++) {
    row_of_tag_[tag_[k]] = k;
    const int i = atom->map(tag_[k]);
    if (i < 0 || i >= nlocal) error->all(FLERR, "verlet/gb300: device atom not found on the host");
    present[i] = 1;
    for (int d = 0; d < 3; d++) {
      atom->x[i][d] = x_[3 * k + d];
      atom->v[i][d] = v_[3 * k + d];
      atom->omega[i][d] = w_[3 * k + d];
      atom->f[i][d] = f_[3 * k + d];
      atom->torque[i][d] = t_[3 * k + d];
    }
  }
  if (n < nlocal) {
    for (int i = nlocal - 1; i >= 0; i--)
      if (!present[i]) {
        atom->avec->copy(nlocal - 1, i, 1);
        present[i] = present[nlocal - 1];
        nlocal--;
      }
    atom->nlocal = nlocal;
    atom->natoms = nlocal;
    atom->nghost = 0;
    atom->map_init();
    atom->map_set();
  }
  natoms_ = atom->natoms;
}

/* moving meshes: the host copy follows the device at output.  Linear motion
   moves every node by the same vector, so the host mesh is translated by the
   difference of one node through the mesh's own move() (which also updates
   its centres and bounding data).  A rotating mesh is turned by the host's
   own mover (FixMoveMesh::initial_integrate, once per step of the
   stretch), which runs the reference's arithmetic on the host copy. */
void VerletGB300::sync_meshes(int nsteps) {
  if (movers_.empty()) return;
  bool linear = false;
  for (size_t k = 0; k < movers_.size(); k++) {
    if (movers_[k]->rotating()) {
      for (int n = 0; n < nsteps; n++) movers_[k]->initial_integrate(0);
    } else {
      linear = true;
    }
  }
  if (!linear) return;
  for (size_t w = 0; w < walls_.size(); w++)
    for (size_t m = 0; m < walls_[w]->mesh_ids().size(); m++) {
      FixMeshSurface *fm =
          dynamic_cast<FixMeshSurface *>(modify->fix[modify->find_fix(walls_[w]->mesh_ids()[m].c_str())]);
      TriMesh *mesh = fm->triMesh();
      const int ntri = mesh->sizeLocal();
      std::vector<double> nodes(9 * (size_t)ntri);
      check(dem_download_mesh_nodes(h_, walls_[w]->device_mesh_ids()[m], &nodes[0]), "dem_download_mesh_nodes");
      if (ntri == 0) continue;
      double host0[3], delta[3];
      mesh->node(0, 0, host0);
      for (int d = 0; d < 3; d++) delta[d] = nodes[d] - host0[d];
      mesh->move(delta);
    }
}

void VerletGB300::add_device_forces() {
  const int nlocal = atom->nlocal;
  for (int i = 0; i < nlocal; i++) {
    const int tg = atom->tag[i];
    const int k = tg < (int)row_of_tag_.size() ? row_of_tag_[tg] : -1;
    if (k < 0) continue;
    for (int d = 0; d < 3; d++) {
      atom->f[i][d] += f_[3 * k + d];
      atom->torque[i][d] += t_[3 * k + d];
    }
  }
}

void VerletGB300::setup() {
  collect_styles();
  if (!h_ || natoms_ != atom->natoms || stamp_ != host_stamp()) create_device();
  // Verlet::setup on the device: pbc + neighbour build with history
  // carry-over + forces without history update
  check(dem_setup(h_), "dem_setup");
  download();
  sync_meshes(0);
  // the reference's own setup for the host side (ghosts, host lists, output
  // at the setup step); pair gran/gb300 copies the device forces in
  Verlet::setup();
  stamp_ = host_stamp();
}

void VerletGB300::setup_minimal(int) {
  error->all(FLERR, "verlet/gb300 does not run minimizations");
}

/* FixInsert::pre_exchange of the insertion step s runs on the host with the
   state the reference gives it.  In Verlet::run the fix is called after the
   initial integration of step s, before pbc and the ghost exchange
   (src/verlet.cpp:298-312), so its overlap checks (FixInsert::load_xnear,
   local and ghost atoms) see the local atoms drifted to step s and the
   ghosts still at step s-1.  The host holds the device state of step s-1:
   the ghosts are built from it, then the local atoms are drifted by the
   reference's own FixNVESphere::initial_integrate, then the fix inserts.
   The new atoms join the device at step s after its initial integration,
   with a rebuild (dem_insert_atoms), as the reference adds them.  The host
   copy of the existing atoms is overwritten by the next download. */
void VerletGB300::insert_due(bigint step) {
  bool drifted = false;
  for (size_t k = 0; k < inserts_.size(); k++) {
    FixInsert *fi = inserts_[k];
    if (!fi->force_reneighbor || fi->next_reneighbor != step) continue;
    // fresh ghosts for the fix's overlap checks
    domain->pbc();
    domain->reset_box();
    comm->setup();
    comm->exchange();
    comm->borders();
    const int n0 = atom->nlocal;
    const bigint ts = update->ntimestep;
    update->ntimestep = step;
    if (!drifted) {
      nve_->FixNVESphere::initial_integrate(0);
      drifted = true;
    }
    fi->pre_exchange();
    update->ntimestep = ts;
    const int k_new = atom->nlocal - n0;
    if (k_new <= 0) continue;
    std::vector<int> tag(k_new), type(k_new);
    std::vector<double> x(3 * (size_t)k_new), v(3 * (size_t)k_new), w(3 * (size_t)k_new), r(k_new), m(k_new);
    for (int q = 0; q < k_new; q++) {
      const int i = n0 + q;
      tag[q] = atom->tag[i];
      type[q] = atom->type[i];
      r[q] = atom->radius[i];
      m[q] = atom->rmass[i];
      for (int d = 0; d < 3; d++) {
        x[3 * q + d] = atom->x[i][d];
        v[3 * q + d] = atom->v[i][d];
        w[3 * q + d] = atom->omega[i][d];
      }
    }
    check(dem_insert_atoms(h_, k_new, &tag[0], &type[0], &x[0], &v[0], &w[0], &r[0], &m[0]), "dem_insert_atoms");
    natoms_ = atom->natoms;
  }
}

void VerletGB300::run(int n) {
  const bigint end = update->ntimestep + n;
  while (update->ntimestep < end) {
    bigint next = end;
    if (output->next > update->ntimestep && output->next < next) next = output->next;
    // stop one step before an insertion step to stage the new atoms
    for (size_t k = 0; k < inserts_.size(); k++)
      if (inserts_[k]->force_reneighbor && inserts_[k]->next_reneighbor > update->ntimestep &&
          inserts_[k]->next_reneighbor - 1 < next)
        next = inserts_[k]->next_reneighbor - 1;
    const int k = (int)(next - update->ntimestep);
    if (k > 0) {
      timer->stamp();
      check(dem_step(h_, k), "dem_step");
      timer->stamp(TIME_PAIR);
      update->ntimestep = next;
      download();
      sync_meshes(k);
      stamp_ = host_stamp();
      if (next == output->next) {
        ev_set(next);
        timer->stamp();
        output->write(next);
        timer->stamp(TIME_OUTPUT);
      }
    }
    if (update->ntimestep < end) {
      insert_due(update->ntimestep + 1);
      stamp_ = host_stamp();
      if (k == 0) {  // the insertion step itself
        timer->stamp();
        check(dem_step(h_, 1), "dem_step");
        timer->stamp(TIME_PAIR);
        update->ntimestep += 1;
        download();
        sync_meshes(1);
        stamp_ = host_stamp();
        if (update->ntimestep == output->next) {
          ev_set(update->ntimestep);
          timer->stamp();
          output->write(update->ntimestep);
          timer->stamp(TIME_OUTPUT);
        }
      }
    }
  }
}

void VerletGB300::cleanup() {
  Verlet::cleanup();
}
