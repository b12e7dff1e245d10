// Context lifecycle, mesh binding, CSR export and host<->device staging of libfcgpu.so.
#include <atomic>
#include <cstring>
#include <string>
#include <vector>

#include "fcg_internal.h"

fcg_context::~fcg_context() {
  for (auto &b : bound_allocs) b.release();
  for (auto &b : stage) b.release();
  dmat.release();
  scratch.release();
  fcg::destroy_krylov(ks);
  fcg::destroy_multi(ms);
  if (switch_ev) cudaEventDestroy(switch_ev);
  if (own_stream) cudaStreamDestroy(own_stream);
}

namespace fcg {

int set_error(fcg_context *c, int status, const std::string &msg) {
  if (c) c->err = msg;
  return status;
}

int cuda_fail(fcg_context *c, cudaError_t e, const char *where) {
  std::string msg = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  cudaGetLastError();  // clear a non-sticky error so that the context stays usable
  return set_error(c, e == cudaErrorMemoryAllocation ? FCG_ERR_NOMEM : FCG_ERR_CUDA, msg);
}

bool is_device_pointer(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int stage_in(fcg_context *c, const void *user, size_t bytes, int slot, bool copy_in, void **dev,
             bool *was_host) {
  if (!user) return set_error(c, FCG_ERR_ARG, "NULL array argument");
  if (is_device_pointer(user)) {
    *dev = const_cast<void *>(user);
    *was_host = false;
    return FCG_OK;
  }
  if ((int)c->stage.size() <= slot) c->stage.resize(slot + 1);
  FCG_CUDA_TRY(c, c->stage[slot].ensure(bytes));
  *dev = c->stage[slot].p;
  *was_host = true;
  if (copy_in && bytes)
    FCG_CUDA_TRY(c, cudaMemcpyAsync(*dev, user, bytes, cudaMemcpyHostToDevice, c->stream));
  return FCG_OK;
}

int stage_out(fcg_context *c, void *user, const void *dev, size_t bytes, bool was_host) {
  if (!was_host || !bytes) return FCG_OK;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
  return FCG_OK;
}

template <class T>
static int upload(fcg_context *c, const T *host, size_t count, const T **out) {
  c->bound_allocs.emplace_back();
  DBuf &b = c->bound_allocs.back();
  FCG_CUDA_TRY(c, b.ensure(count * sizeof(T)));
  if (count) FCG_CUDA_TRY(c, cudaMemcpy(b.p, host, count * sizeof(T), cudaMemcpyHostToDevice));
  *out = (const T *)b.p;
  return FCG_OK;
}

template <class T>
static int host_copy(fcg_context *c, const T *user, size_t count, std::vector<T> &out) {
  out.resize(count);
  if (!count) return FCG_OK;
  if (is_device_pointer(user)) {
    FCG_CUDA_TRY(c, cudaMemcpy(out.data(), user, count * sizeof(T), cudaMemcpyDeviceToHost));
  } else {
    std::memcpy(out.data(), user, count * sizeof(T));
  }
  return FCG_OK;
}

}  // namespace fcg

using namespace fcg;

extern "C" int fcg_abi_version(void) { return FCG_ABI_VERSION; }

extern "C" const char *fcg_status_string(int s) {
  switch (s) {
    case FCG_OK: return "ok";
    case FCG_ERR_ARG: return "invalid argument";
    case FCG_ERR_STATE: return "invalid call order";
    case FCG_ERR_CUDA: return "CUDA error";
    case FCG_ERR_INDEX: return "mesh index out of range";
    case FCG_ERR_PIVOT: return "zero or non-finite pivot";
    case FCG_ERR_STALL: return "iteration stalled";
    case FCG_ERR_TIMEOUT: return "device wait timed out";
    case FCG_ERR_UNSUPPORTED: return "unsupported feature";
    case FCG_ERR_NOMEM: return "device out of memory";
    case FCG_ERR_NONFINITE: return "non-finite value";
    default: return "unknown status";
  }
}

extern "C" const char *fcg_last_error(const fcg_context *c) { return c ? c->err.c_str() : ""; }

extern "C" int fcg_create(fcg_context **out, int device) {
  if (!out) return FCG_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FCG_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return FCG_ERR_ARG;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FCG_ERR_CUDA;
  if (prop.major * 10 + prop.minor < 100) return FCG_ERR_CUDA;  // built for sm_103a only
  if (cudaSetDevice(device) != cudaSuccess) return FCG_ERR_CUDA;
  static std::atomic<unsigned long long> next_uid{1};
  fcg_context *c = new fcg_context();
  c->uid = next_uid++;
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return FCG_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return FCG_OK;
}

extern "C" int fcg_destroy(fcg_context *c) {
  if (!c) return FCG_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  delete c;
  return FCG_OK;
}

// Work queued later on the new stream is ordered after work already queued on the old
// one (an event, no host wait); the old stream must still exist.
extern "C" int fcg_set_stream(fcg_context *c, void *s) {
  if (!c) return FCG_ERR_ARG;
  cudaStream_t ns = s ? (cudaStream_t)s : c->own_stream;
  if (ns != c->stream) {
    FCG_CUDA_TRY(c, cudaSetDevice(c->device));
    if (!c->switch_ev)
      FCG_CUDA_TRY(c, cudaEventCreateWithFlags(&c->switch_ev, cudaEventDisableTiming));
    FCG_CUDA_TRY(c, cudaEventRecord(c->switch_ev, c->stream));
    FCG_CUDA_TRY(c, cudaStreamWaitEvent(ns, c->switch_ev, 0));
  }
  c->stream = ns;
  return FCG_OK;
}

extern "C" int fcg_synchronize(fcg_context *c) {
  if (!c) return FCG_ERR_ARG;
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_mesh_sizes(const fcg_context *c, int *n, int *nf, int *nin, long long *nnz,
                              int *ntot) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return FCG_ERR_STATE;
  if (n) *n = c->n;
  if (nf) *nf = c->nf;
  if (nin) *nin = c->nin;
  if (nnz) *nnz = c->nnz;
  if (ntot) *ntot = c->ntot;
  return FCG_OK;
}

extern "C" int fcg_bind_mesh(fcg_context *c, const fcg_mesh_desc *m) {
  if (!c || !m) return FCG_ERR_ARG;
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  if (m->numCells <= 0 || m->numFaces <= 0 || m->numInnerFaces < 0 ||
      m->numInnerFaces > m->numFaces)
    return set_error(c, FCG_ERR_ARG, "mesh sizes out of range");
  if (m->noc != 0)
    return set_error(c, FCG_ERR_UNSUPPORTED, "O-C grid cuts (noc > 0) are not supported");
  const double *dp[] = {m->arx, m->ary, m->arz, m->xf, m->yf, m->zf, m->xc, m->yc, m->zc, m->vol};
  for (const double *p : dp)
    if (!p) return set_error(c, FCG_ERR_ARG, "NULL geometry array in fcg_mesh_desc");
  if (!m->owner || (m->numInnerFaces > 0 && (!m->neighbour || !m->facint)))
    return set_error(c, FCG_ERR_ARG, "NULL connectivity array in fcg_mesh_desc");
  // Release a previous mesh.
  for (auto &b : c->bound_allocs) b.release();
  c->bound_allocs.clear();
  c->bound = false;
  c->dmat_ready = false;

  const int n = m->numCells, nf = m->numFaces, nin = m->numInnerFaces, nb = nf - nin;
  int cnt[B_NTYPES] = {m->ninl, m->nout, m->nsym, m->nwal, m->npru};
  int fst[B_NTYPES] = {m->iInletFacesStart, m->iOutletFacesStart, m->iSymmetryFacesStart,
                       m->iWallFacesStart, m->iPressOutletFacesStart};
  int bst[B_NTYPES];
  long long acc = n;
  for (int t = 0; t < B_NTYPES; ++t) {
    if (cnt[t] < 0) return set_error(c, FCG_ERR_ARG, "negative boundary count");
    bst[t] = (int)acc;  // mesh_geometry_and_topology.f90:593-605, 0-based
    acc += cnt[t];
  }
  if (acc - n > nb) return set_error(c, FCG_ERR_INDEX, "boundary counts exceed the boundary faces");

  // Host copies of the connectivity (the caller may hand device arrays).
  fcg_mesh_desc hm = *m;
  std::vector<int> own, nei;
  int rc = host_copy(c, m->owner, nf, own);
  if (rc) return rc;
  if ((rc = host_copy(c, m->neighbour, nin, nei))) return rc;
  hm.owner = own.data();
  hm.neighbour = nei.data();
  HostTopology t;
  std::string err;
  if ((rc = validate_topology(hm, cnt, fst, err))) return set_error(c, rc, err);
  // The CSR and slot maps by the GPU kernels of fcg_csr_build_gpu (identical to the host
  // construction, which is a sequential scatter over the faces), the rest on the host.
  if ((long long)n + 2LL * nin <= 0x7fffffffLL) {
    t.ioffset.resize(n + 1);
    t.ja.resize((size_t)n + 2 * (size_t)nin);
    t.diag.resize(n);
    t.slot_pn.resize(nin);
    t.slot_np.resize(nin);
    if ((rc = fcg_csr_build_gpu(c, n, nin, own.data(), nei.data(), t.ioffset.data(), t.ja.data(),
                                t.diag.data(), t.slot_pn.data(), t.slot_np.data())))
      return rc;
    rc = build_topology(hm, cnt, fst, bst, t, err, true);
  } else {
    rc = build_topology(hm, cnt, fst, bst, t, err);
  }
  if (rc) return set_error(c, rc, err);

  c->n = n;
  c->nf = nf;
  c->nin = nin;
  c->nb = nb;
  c->ntot = n + nb;
  c->nnz = (long long)t.ja.size();
  std::memcpy(c->cnt, cnt, sizeof cnt);
  std::memcpy(c->fst, fst, sizeof fst);
  std::memcpy(c->bst, bst, sizeof bst);

  MeshView &v = c->mv;
  std::memset(&v, 0, sizeof v);
  v.n = n;
  v.nf = nf;
  v.nin = nin;
  v.ntot = c->ntot;
  v.nnz = c->nnz;
  std::vector<int> own0(own), nei0(nei);
  for (auto &x : own0) x -= 1;
  for (auto &x : nei0) x -= 1;
#define UP(dst, src, count)                                  \
  do {                                                       \
    if ((rc = upload(c, (src), (size_t)(count), &(dst)))) return rc; \
  } while (0)
  UP(v.owner, own0.data(), nf);
  UP(v.neighbour, nei0.data(), nin);
  // Geometry may be host or device; stage it through host vectors.
  std::vector<double> tmp;
  const double *src_f[] = {m->arx, m->ary, m->arz, m->xf, m->yf, m->zf};
  const double **dst_f[] = {&v.arx, &v.ary, &v.arz, &v.xf, &v.yf, &v.zf};
  for (int i = 0; i < 6; ++i) {
    if ((rc = host_copy(c, src_f[i], nf, tmp))) return rc;
    UP(*dst_f[i], tmp.data(), nf);
  }
  const double *src_c[] = {m->xc, m->yc, m->zc, m->vol};
  const double **dst_c[] = {&v.xc, &v.yc, &v.zc, &v.vol};
  for (int i = 0; i < 4; ++i) {
    if ((rc = host_copy(c, src_c[i], n, tmp))) return rc;
    UP(*dst_c[i], tmp.data(), n);
  }
  if ((rc = host_copy(c, m->facint, nin, tmp))) return rc;
  UP(v.facint, tmp.data(), nin);

  std::vector<int> io0(t.ioffset), ja0(t.ja), dg0(t.diag), spn0(t.slot_pn), snp0(t.slot_np);
  for (auto &x : io0) x -= 1;
  for (auto &x : ja0) x -= 1;
  for (auto &x : dg0) x -= 1;
  for (auto &x : spn0) x -= 1;
  for (auto &x : snp0) x -= 1;
  UP(v.ioffset, io0.data(), n + 1);
  UP(v.ja, ja0.data(), ja0.size());
  UP(v.diag, dg0.data(), n);
  UP(v.slot_pn, spn0.data(), nin);
  UP(v.slot_np, snp0.data(), nin);
  UP(c->tpos, t.tpos.data(), t.tpos.size());
  UP(v.cf_ptr, t.cf_ptr.data(), t.cf_ptr.size());
  UP(v.cf_ent, t.cf_ent.data(), t.cf_ent.size());
  UP(v.cf_slot, t.cf_slot.data(), t.cf_slot.size());
  UP(v.cb_ptr, t.cb_ptr.data(), t.cb_ptr.size());
  UP(v.cb_face, t.cb_face.data(), t.cb_face.size());
  UP(v.cb_slot, t.cb_slot.data(), t.cb_slot.size());
  UP(v.cb_type, t.cb_type.data(), t.cb_type.size());
  UP(v.cbf_ptr, t.cbf_ptr.data(), t.cbf_ptr.size());
  UP(v.cbf_face, t.cbf_face.data(), t.cbf_face.size());

  SellView &s = c->sv;
  s.nslices = (int)t.sell_width.size();
  UP(s.ptr, t.sell_ptr.data(), t.sell_ptr.size());
  UP(s.width, t.sell_width.data(), t.sell_width.size());
  UP(s.kind, t.sell_kind.data(), t.sell_kind.size());
  UP(s.offp, t.sell_offp.data(), t.sell_offp.size());
  UP(s.off, t.sell_off.data(), t.sell_off.size());
  UP(s.src, t.sell_src.data(), t.sell_src.size());
  c->sell_maxw = t.sell_maxw;
  c->sell_len = t.sell_ptr.back();
  c->sell_nuniform = t.sell_nuniform;

  const int *rows;
  c->lf.ptr = t.lf_ptr;
  c->lf.count = (int)t.lf_ptr.size() - 1;
  UP(rows, t.lf_rows.data(), t.lf_rows.size());
  c->lf.rows = const_cast<int *>(rows);
  c->lb.ptr = t.lb_ptr;
  c->lb.count = (int)t.lb_ptr.size() - 1;
  UP(rows, t.lb_rows.data(), t.lb_rows.size());
  c->lb.rows = const_cast<int *>(rows);
  {
    auto padded = [](const std::vector<int> &ptr, const std::vector<int> &rs) {
      std::vector<int> out;
      out.reserve(rs.size() + 32 * ptr.size());
      for (size_t l = 0; l + 1 < ptr.size(); ++l) {
        out.insert(out.end(), rs.begin() + ptr[l], rs.begin() + ptr[l + 1]);
        while (out.size() % 32) out.push_back(-1);
      }
      return out;
    };
    std::vector<int> pf = padded(t.lf_ptr, t.lf_rows), pb = padded(t.lb_ptr, t.lb_rows);
    UP(rows, pf.data(), pf.size());
    c->lf.pad = const_cast<int *>(rows);
    c->lf.pad_len = (int)pf.size();
    UP(rows, pb.data(), pb.size());
    c->lb.pad = const_cast<int *>(rows);
    c->lb.pad_len = (int)pb.size();
  }
#undef UP

  c->h_ioffset.swap(t.ioffset);
  c->h_ja.swap(t.ja);
  c->h_diag.swap(t.diag);
  c->h_slot_pn.swap(t.slot_pn);
  c->h_slot_np.swap(t.slot_np);
  c->bound = true;
  c->bind_gen++;
  return FCG_OK;
}

extern "C" int fcg_create_csr(fcg_context *c, int *ioffset, int *ja, int *diag, int *slot_pn,
                              int *slot_np) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_create_csr before fcg_bind_mesh");
  struct {
    int *dst;
    const std::vector<int> *src;
  } outs[] = {{ioffset, &c->h_ioffset}, {ja, &c->h_ja}, {diag, &c->h_diag},
              {slot_pn, &c->h_slot_pn}, {slot_np, &c->h_slot_np}};
  for (auto &o : outs) {
    if (!o.dst || o.src->empty()) continue;
    size_t bytes = o.src->size() * sizeof(int);
    if (is_device_pointer(o.dst)) {
      FCG_CUDA_TRY(c, cudaMemcpy(o.dst, o.src->data(), bytes, cudaMemcpyHostToDevice));
    } else {
      std::memcpy(o.dst, o.src->data(), bytes);
    }
  }
  return FCG_OK;
}
