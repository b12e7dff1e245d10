// Context lifecycle, mesh binding, CSR export and host<->device staging of libfcgpu.so.
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fcg_internal.h"

fcg_context::~fcg_context() {
  for (auto &b : bound_allocs) b.release();
  for (auto &b : stage) b.release();
  dmat.release();
  fgeo.release();
  bgeo.release();
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

// A bound device copy of a caller array that may be host or device memory, copied in
// one transfer (no host staging).
template <class T>
static int upload_any(fcg_context *c, const T *user, size_t count, const T **out) {
  c->bound_allocs.emplace_back();
  DBuf &b = c->bound_allocs.back();
  FCG_CUDA_TRY(c, b.ensure(count * sizeof(T)));
  if (count)
    FCG_CUDA_TRY(c, cudaMemcpy(b.p, user, count * sizeof(T),
                               is_device_pointer(user) ? cudaMemcpyDeviceToDevice
                                                       : cudaMemcpyHostToDevice));
  *out = (const T *)b.p;
  return FCG_OK;
}

// The O-C pairs of a mesh (mesh_geometry_and_topology.f90:800-845): the two cells of
// every pair from the owners of its faces, every cell's pair entries in pair order (the
// left cell's before the right cell's within a pair, as the reference's loops update
// ijl(i) before ijr(i)), and foc / srdoc computed on the device (oc_geometry).
static int bind_oc(fcg_context *c, const fcg_mesh_desc &m, const std::vector<int> &own) {
  const int noc = m.noc, n = m.numCells;
  std::vector<int> fl, fr;
  int rc;
  if ((rc = host_copy(c, m.ijlFace, (size_t)noc, fl)) || (rc = host_copy(c, m.ijrFace, (size_t)noc, fr)))
    return rc;
  std::vector<int> l(noc), r(noc);
  for (int i = 0; i < noc; ++i) {
    if (fl[i] <= m.numInnerFaces || fl[i] > m.numFaces || fr[i] <= m.numInnerFaces ||
        fr[i] > m.numFaces)
      return set_error(c, FCG_ERR_INDEX, "an O-C pair names a face that is not a boundary face");
    fl[i] -= 1;
    fr[i] -= 1;
    l[i] = own[fl[i]] - 1;
    r[i] = own[fr[i]] - 1;
    if (l[i] == r[i]) return set_error(c, FCG_ERR_INDEX, "an O-C pair couples a cell to itself");
  }
  std::vector<int> ptr((size_t)n + 1, 0), col(2 * (size_t)noc), vix(2 * (size_t)noc);
  for (int i = 0; i < noc; ++i) {
    ++ptr[(size_t)l[i] + 1];
    ++ptr[(size_t)r[i] + 1];
  }
  for (int k = 0; k < n; ++k) ptr[(size_t)k + 1] += ptr[k];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int i = 0; i < noc; ++i) {
    int e = fill[l[i]]++;  // row ijl(i): ar(i) * x(ijr(i))
    col[e] = r[i];
    vix[e] = i;
    e = fill[r[i]]++;  // row ijr(i): al(i) * x(ijl(i))
    col[e] = l[i];
    vix[e] = noc + i;
  }
  MeshView &v = c->mv;
  if ((rc = upload(c, l.data(), (size_t)noc, &v.oc_l)) ||
      (rc = upload(c, r.data(), (size_t)noc, &v.oc_r)) ||
      (rc = upload(c, fl.data(), (size_t)noc, &v.oc_fl)) ||
      (rc = upload(c, fr.data(), (size_t)noc, &v.oc_fr)) ||
      (rc = upload(c, ptr.data(), ptr.size(), &v.oc_cptr)) ||
      (rc = upload(c, col.data(), col.size(), &v.oc_col)) ||
      (rc = upload(c, vix.data(), vix.size(), &v.oc_vix)))
    return rc;
  v.noc = noc;
  v.ncyc = m.ncyc;
  v.oc_start = m.iOCFacesStart;
  return oc_geometry(c);
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
  if (m->noc < 0 || m->ncyc < 0 || m->ncyc > m->noc)
    return set_error(c, FCG_ERR_ARG, "noc or ncyc out of range");
  if (m->noc > 0 && (!m->ijlFace || !m->ijrFace))
    return set_error(c, FCG_ERR_ARG, "noc > 0 without ijlFace / ijrFace");
  // faces iOCFacesStart + 1 .. + noc give the pairs' areas (fvm_laplacian.f90:70); with
  // cyclic pairs only the start stays 0, as the reference leaves it
  if (m->noc > 0 && (m->iOCFacesStart < 0 || (long long)m->iOCFacesStart + m->noc > m->numFaces))
    return set_error(c, FCG_ERR_INDEX, "iOCFacesStart + noc is outside the faces");
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
  c->fgeo_ready = false;
  c->bgeo_ready = false;

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
  // The topology is built on the device (bind_topology_device), identical to the host
  // construction, which FCG_TOPOLOGY=host selects instead.
  const char *te = std::getenv("FCG_TOPOLOGY");
  const bool host_topo =
      (te && std::string(te) == "host") || (long long)n + 2LL * nin > 0x7fffffffLL;
  if (host_topo && (rc = build_topology(hm, cnt, fst, bst, t, err))) return set_error(c, rc, err);

  c->n = n;
  c->nf = nf;
  c->nin = nin;
  c->nb = nb;
  c->ntot = n + nb;
  c->nnz = host_topo ? (long long)t.ja.size() : (long long)n + 2LL * nin;
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
#define UP(dst, src, count)                                  \
  do {                                                       \
    if ((rc = upload(c, (src), (size_t)(count), &(dst)))) return rc; \
  } while (0)
  // owner / neighbour: the 1-based host copies, made 0-based on the device
  if ((rc = upload_any(c, own.data(), (size_t)nf, &v.owner)) ||
      (rc = upload_any(c, nei.data(), (size_t)nin, &v.neighbour)))
    return rc;
  if ((rc = to_zero_based(c, const_cast<int *>(v.owner), nf)) ||
      (rc = to_zero_based(c, const_cast<int *>(v.neighbour), nin)))
    return rc;
  // geometry, host or device, copied as it is
  const double *src_f[] = {m->arx, m->ary, m->arz, m->xf, m->yf, m->zf};
  const double **dst_f[] = {&v.arx, &v.ary, &v.arz, &v.xf, &v.yf, &v.zf};
  for (int i = 0; i < 6; ++i)
    if ((rc = upload_any(c, src_f[i], (size_t)nf, dst_f[i]))) return rc;
  const double *src_c[] = {m->xc, m->yc, m->zc, m->vol};
  const double **dst_c[] = {&v.xc, &v.yc, &v.zc, &v.vol};
  for (int i = 0; i < 4; ++i)
    if ((rc = upload_any(c, src_c[i], (size_t)n, dst_c[i]))) return rc;
  if ((rc = upload_any(c, m->facint, (size_t)nin, &v.facint))) return rc;
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));

  if (!host_topo) {
    if ((rc = bind_topology_device(c, v.owner, v.neighbour, own, cnt, fst, bst, err)))
      return err.empty() ? rc : set_error(c, rc, err);
  } else {
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
  }
#undef UP

  if (host_topo) {
    c->topo.clear();
    {
      auto rec = [&](const void *p, size_t bytes) { c->topo.emplace_back(p, bytes); };
      rec(v.ioffset, sizeof(int) * (n + 1));
      rec(v.ja, sizeof(int) * t.ja.size());
      rec(v.diag, sizeof(int) * n);
      rec(v.slot_pn, sizeof(int) * nin);
      rec(v.slot_np, sizeof(int) * nin);
      rec(c->tpos, sizeof(int) * t.tpos.size());
      rec(v.cf_ptr, sizeof(int) * t.cf_ptr.size());
      rec(v.cf_ent, sizeof(int) * t.cf_ent.size());
      rec(v.cf_slot, sizeof(int) * t.cf_slot.size());
      rec(v.cb_ptr, sizeof(int) * t.cb_ptr.size());
      rec(v.cb_face, sizeof(int) * t.cb_face.size());
      rec(v.cb_slot, sizeof(int) * t.cb_slot.size());
      rec(v.cb_type, sizeof(int) * t.cb_type.size());
      rec(v.cbf_ptr, sizeof(int) * t.cbf_ptr.size());
      rec(v.cbf_face, sizeof(int) * t.cbf_face.size());
      rec(c->sv.ptr, sizeof(long long) * t.sell_ptr.size());
      rec(c->sv.width, sizeof(int) * t.sell_width.size());
      rec(c->sv.kind, sizeof(int) * t.sell_kind.size());
      rec(c->sv.offp, sizeof(int) * t.sell_offp.size());
      rec(c->sv.off, sizeof(int) * t.sell_off.size());
      rec(c->sv.src, sizeof(int) * t.sell_src.size());
      rec(c->lf.rows, sizeof(int) * t.lf_rows.size());
      rec(c->lb.rows, sizeof(int) * t.lb_rows.size());
      rec(c->lf.pad, sizeof(int) * c->lf.pad_len);
      rec(c->lb.pad, sizeof(int) * c->lb.pad_len);
    }
  }
  if (m->noc > 0 && (rc = bind_oc(c, *m, own))) return rc;
  if ((rc = detect_hex_block(c))) return rc;
  c->bound = true;
  c->bind_gen++;
  return FCG_OK;
}

extern "C" int fcg_topology_digest(fcg_context *c, unsigned long long *digest) {
  if (!c || !digest) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_topology_digest before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  unsigned long long h = 1469598103934665603ULL;  // FNV-1a, 64 bit
  auto mix = [&](const unsigned char *b, size_t nb) {
    for (size_t i = 0; i < nb; ++i) {
      h ^= b[i];
      h *= 1099511628211ULL;
    }
  };
  std::vector<unsigned char> buf;
  for (const auto &a : c->topo) {
    buf.resize(a.second);
    if (a.second) FCG_CUDA_TRY(c, cudaMemcpy(buf.data(), a.first, a.second, cudaMemcpyDeviceToHost));
    const unsigned long long len = a.second;
    mix(reinterpret_cast<const unsigned char *>(&len), sizeof len);
    mix(buf.data(), buf.size());
  }
  for (const auto *lv : {&c->lf, &c->lb})
    mix(reinterpret_cast<const unsigned char *>(lv->ptr.data()), sizeof(int) * lv->ptr.size());
  *digest = h;
  return FCG_OK;
}

extern "C" int fcg_create_csr(fcg_context *c, int *ioffset, int *ja, int *diag, int *slot_pn,
                              int *slot_np) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_create_csr before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  // the bound CSR is 0-based on the device; the reference's arrays are 1-based
  struct {
    int *dst;
    const int *src;
    size_t count;
  } outs[] = {{ioffset, c->mv.ioffset, (size_t)c->n + 1}, {ja, c->mv.ja, (size_t)c->nnz},
              {diag, c->mv.diag, (size_t)c->n}, {slot_pn, c->mv.slot_pn, (size_t)c->nin},
              {slot_np, c->mv.slot_np, (size_t)c->nin}};
  std::vector<int> tmp;
  for (auto &o : outs) {
    if (!o.dst || !o.count) continue;
    tmp.resize(o.count);
    FCG_CUDA_TRY(c, cudaMemcpy(tmp.data(), o.src, o.count * sizeof(int), cudaMemcpyDeviceToHost));
    for (auto &x : tmp) x += 1;
    if (is_device_pointer(o.dst)) {
      FCG_CUDA_TRY(c, cudaMemcpy(o.dst, tmp.data(), o.count * sizeof(int), cudaMemcpyHostToDevice));
    } else {
      std::memcpy(o.dst, tmp.data(), o.count * sizeof(int));
    }
  }
  return FCG_OK;
}
