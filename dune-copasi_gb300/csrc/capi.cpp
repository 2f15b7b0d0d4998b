// extern "C" boundary (include/dcgpu.h).  Exceptions are caught here and turned into
// status codes; the message is kept per thread for dc_last_error().
#include <cstring>
#include <memory>
#include <string>

#include "../../include/dcgpu.h"
#include "amg.hpp"
#include "graph.hpp"
#include "handle.hpp"
#include "mcolor.hpp"

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F&& f) {
  try {
    g_last_error.clear();
    return f();
  } catch (const dcgpu::ConfigError& e) {
    g_last_error = e.what();
    return DC_ERR_CONFIG;
  } catch (const dcgpu::CudaError& e) {
    g_last_error = e.what();
    return DC_ERR_CUDA;
  } catch (const dcgpu::StepFailure& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return DC_ERR_ARGUMENT;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return DC_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown error";
    return DC_ERR_INTERNAL;
  }
}

}  // namespace

extern "C" {

const char* dc_last_error(void) { return g_last_error.c_str(); }

int dc_model_create(const char* ini_text, const char* overrides, dc_model** out) {
  return guarded([&] {
    if (!ini_text || !out) throw std::invalid_argument("null argument");
    *out = nullptr;
    int dev_count = 0;
    dcgpu::cuda_check(cudaGetDeviceCount(&dev_count), "cudaGetDeviceCount");
    if (dev_count == 0) throw dcgpu::CudaError("no CUDA device");
    auto m = std::make_unique<dc_model>();
    dcgpu::cuda_check(cudaGetDevice(&m->device), "cudaGetDevice");
    dcgpu::cuda_check(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    m->model = std::make_unique<dcgpu::Model>(ini_text, overrides ? overrides : "");
    m->solver = std::make_unique<dcgpu::Solver>(*m->model, m->stream);
    dc_noalloc_prepare(m->device);
    *out = m.release();
    return DC_OK;
  });
}

int dc_config_get(const dc_model* model, const char* key, char* buf, size_t len) {
  return guarded([&] {
    if (!model || !key || !buf || len == 0) throw std::invalid_argument("null argument");
    const auto& cfg = model->model->cfg;
    if (!cfg.has_key(key)) throw dcgpu::ConfigError(std::string("no configuration key '") + key + "'");
    const std::string v = cfg.get(key, "");
    std::strncpy(buf, v.c_str(), len - 1);
    buf[len - 1] = '\0';
    return DC_OK;
  });
}

int dc_model_destroy(dc_model* model) {
  return guarded([&] {
    if (!model) return DC_OK;
    cudaStream_t s = model->stream;
    if (s) cudaStreamSynchronize(s);
    model->solver.reset();
    model->model.reset();
    if (s) cudaStreamDestroy(s);
    delete model;
    return DC_OK;
  });
}

int dc_model_info_get(const dc_model* model, dc_model_info* info) {
  return guarded([&] {
    if (!model || !info) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    info->dim = m.dim;
    info->n_species = static_cast<int32_t>(m.species.size());
    info->n_compartments = static_cast<int32_t>(m.comp_names.size());
    info->block_size = m.bs;
    info->n_vertices = m.mesh.nv;
    info->n_elements = m.mesh.ne;
    info->n_dof = m.ndof;
    info->n_block_rows = m.nnodes;
    info->n_blocks = m.nnzb();
    return DC_OK;
  });
}

int dc_species_name(const dc_model* model, int32_t species, char* buf, size_t len) {
  return guarded([&] {
    if (!model || !buf) throw std::invalid_argument("null argument");
    const auto& sp = model->model->species;
    if (species < 0 || species >= static_cast<int32_t>(sp.size())) throw std::invalid_argument("species index out of range");
    const std::string& n = sp[species].name;
    if (len < n.size() + 1) throw std::invalid_argument("buffer too small");
    std::memcpy(buf, n.c_str(), n.size() + 1);
    return DC_OK;
  });
}

int dc_species_size(const dc_model* model, int32_t species, int64_t* n_vertices) {
  return guarded([&] {
    if (!model || !n_vertices) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    if (species < 0 || species >= static_cast<int32_t>(m.species.size())) throw std::invalid_argument("species index out of range");
    *n_vertices = static_cast<int64_t>(m.comp_vertices[m.species[species].comp].size());
    return DC_OK;
  });
}

int dc_species_vertices(const dc_model* model, int32_t species, int64_t* vertex_ids, size_t n) {
  return guarded([&] {
    if (!model || !vertex_ids) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    if (species < 0 || species >= static_cast<int32_t>(m.species.size())) throw std::invalid_argument("species index out of range");
    const auto& v = m.comp_vertices[m.species[species].comp];
    if (n != v.size()) throw std::invalid_argument("size mismatch");
    for (size_t k = 0; k < n; ++k) vertex_ids[k] = v[k];
    return DC_OK;
  });
}

int dc_vertex_coords(const dc_model* model, double* coords, size_t n) {
  return guarded([&] {
    if (!model || !coords) throw std::invalid_argument("null argument");
    const auto& c = model->model->mesh.coords;
    if (n != c.size()) throw std::invalid_argument("size mismatch");
    std::memcpy(coords, c.data(), n * sizeof(double));
    return DC_OK;
  });
}

int dc_constraints(const dc_model* model, int64_t* dofs, double* values, size_t n, size_t* n_out) {
  return guarded([&] {
    if (!model || !n_out) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    *n_out = static_cast<size_t>(m.n_constraints);
    if (!dofs && !values) return DC_OK;
    if (n != static_cast<size_t>(m.n_constraints)) throw std::invalid_argument("size mismatch");
    for (int64_t k = 0; k < m.n_constraints; ++k) {
      const int64_t node = m.cons_idx[k] / m.bs;
      const int local = static_cast<int>(m.cons_idx[k] % m.bs);
      int c = 0;
      while (node >= m.comp_node_offset[c + 1]) ++c;
      if (dofs) dofs[k] = m.ref_dof(c, static_cast<int32_t>(node - m.comp_node_offset[c]), local);
      if (values) values[k] = m.cons_val[k];
    }
    return DC_OK;
  });
}

int dc_state_set_initial(dc_model* model) {
  return guarded([&] {
    if (!model) throw std::invalid_argument("null argument");
    auto& m = *model->model;
    model->solver->set_state(m.initial_state(), m.cfg.sub("model").get_double("time_step_operator.time_begin", 0.0));
    return DC_OK;
  });
}

int dc_state_get(const dc_model* model, double* host_out, size_t n) {
  return guarded([&] {
    if (!model || !host_out) throw std::invalid_argument("null argument");
    if (static_cast<int64_t>(n) != model->model->ndof) throw std::invalid_argument("size mismatch");
    model->solver->get_state(host_out, static_cast<int64_t>(n));
    return DC_OK;
  });
}

int dc_write_vtk(const dc_model* model, const char* path, int append) {
  return guarded([&] {
    if (!model || !path) throw std::invalid_argument("null argument");
    model->model->write_vtk(model->solver->get_state(), model->solver->time(), path, append != 0);
    return DC_OK;
  });
}

int dc_state_set(dc_model* model, const double* host_in, size_t n, double time) {
  return guarded([&] {
    if (!model || !host_in) throw std::invalid_argument("null argument");
    if (static_cast<int64_t>(n) != model->model->ndof) throw std::invalid_argument("size mismatch");
    model->solver->set_state(host_in, static_cast<int64_t>(n), time);
    return DC_OK;
  });
}

int dc_state_get_species(const dc_model* model, int32_t species, double* host_out, size_t n) {
  return guarded([&] {
    if (!model || !host_out) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    if (species < 0 || species >= static_cast<int32_t>(m.species.size())) throw std::invalid_argument("species index out of range");
    const auto& sp = m.species[species];
    const auto& verts = m.comp_vertices[sp.comp];
    if (n != verts.size()) throw std::invalid_argument("size mismatch");
    auto v = model->solver->get_state();
    for (size_t k = 0; k < n; ++k) host_out[k] = v[m.ref_dof(sp.comp, static_cast<int32_t>(k), sp.local)];
    return DC_OK;
  });
}

int dc_state_time(const dc_model* model, double* time) {
  return guarded([&] {
    if (!model || !time) throw std::invalid_argument("null argument");
    *time = model->solver->time();
    return DC_OK;
  });
}

int dc_step(dc_model* model, double* dt, dc_step_info* info) {
  return guarded([&] {
    if (!model || !dt) throw std::invalid_argument("null argument");
    auto& s = *model->solver;
    const auto before = s.stats;
    double used = 0.0;
    cudaEvent_t e0, e1;
    dcgpu::cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
    dcgpu::cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
    dcgpu::cuda_check(cudaEventRecord(e0, model->stream), "cudaEventRecord");
    int st = s.do_step(*dt, &used);
    dcgpu::cuda_check(cudaEventRecord(e1, model->stream), "cudaEventRecord");
    dcgpu::cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
    float ms = 0.0f;
    dcgpu::cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (info) {
      info->device_ms = ms;
      info->time = s.time();
      info->dt_used = used;
      info->newton_iterations = static_cast<int32_t>(s.stats.newton_iterations - before.newton_iterations);
      info->linear_iterations = static_cast<int32_t>(s.stats.linear_iterations - before.linear_iterations);
      info->failed_attempts = static_cast<int32_t>(s.stats.failed_steps - before.failed_steps);
      info->status = st;
    }
    if (st != DC_OK) g_last_error = "time step failed";
    return st;
  });
}

int dc_evolve(dc_model* model, double t_end, double* dt, dc_callback cb, void* user) {
  return guarded([&] {
    if (!model || !dt) throw std::invalid_argument("null argument");
    int st = model->solver->evolve(t_end, *dt, [&](double t) {
      if (cb) cb(model, t, user);
    });
    if (st != DC_OK) g_last_error = "evolve failed";
    return st;
  });
}

int dc_assemble(dc_model* model, const double* x, double t, double cm, double ca, double* r, double* jac_values,
                size_t n_jac_values) {
  return guarded([&] {
    if (!model || !x) throw std::invalid_argument("null argument");
    auto& m = *model->model;
    const int64_t n = m.nnodes * m.bs;
    const int64_t nj = m.nnzb() * m.bs * m.bs;
    if (jac_values && static_cast<int64_t>(n_jac_values) != nj) throw std::invalid_argument("jacobian size mismatch");
    std::vector<double> blk;
    m.to_blocked(std::vector<double>(x, x + m.ndof), blk);
    if (model->scratch_x.size() != static_cast<size_t>(n)) model->scratch_x.resize(n);
    if (model->scratch_r.size() != static_cast<size_t>(n)) model->scratch_r.resize(n);
    if (jac_values && model->scratch_j.size() != static_cast<size_t>(nj)) model->scratch_j.resize(nj);
    cudaStream_t s = model->stream;
    dcgpu::cuda_check(cudaMemcpyAsync(model->scratch_x.get(), blk.data(), n * sizeof(double), cudaMemcpyHostToDevice, s), "copy");
    dcgpu::cuda_check(cudaMemsetAsync(model->scratch_r.get(), 0, n * sizeof(double), s), "memset");
    if (jac_values) dcgpu::cuda_check(cudaMemsetAsync(model->scratch_j.get(), 0, nj * sizeof(double), s), "memset");
    int mode = (r ? 1 : 0) | (jac_values ? 2 : 0);
    if (mode) m.assemble(model->scratch_x.get(), t, cm, ca, r ? model->scratch_r.get() : nullptr,
                         jac_values ? model->scratch_j.get() : nullptr, mode, s);
    dcgpu::cuda_check(cudaStreamSynchronize(s), "assemble");
    dcgpu::cuda_check(cudaGetLastError(), "assemble");
    if (r) {
      std::vector<double> rb(n), rr;
      dcgpu::cuda_check(cudaMemcpy(rb.data(), model->scratch_r.get(), n * sizeof(double), cudaMemcpyDeviceToHost), "copy");
      m.from_blocked(rb, rr);
      std::memcpy(r, rr.data(), m.ndof * sizeof(double));
    }
    if (jac_values)
      dcgpu::cuda_check(cudaMemcpy(jac_values, model->scratch_j.get(), nj * sizeof(double), cudaMemcpyDeviceToHost), "copy");
    return DC_OK;
  });
}

int dc_jacobian_apply(dc_model* model, const double* x, double t, double cm, double ca, const double* v, double* y) {
  return guarded([&] {
    if (!model || !x || !v || !y) throw std::invalid_argument("null argument");
    auto& m = *model->model;
    const int64_t n = m.nnodes * m.bs;
    std::vector<double> bx, bv;
    m.to_blocked(std::vector<double>(x, x + m.ndof), bx);
    m.to_blocked(std::vector<double>(v, v + m.ndof), bv);
    dcgpu::DeviceBuffer<double> dx, dv, dy(static_cast<size_t>(n));
    dx.upload(bx);
    dv.upload(bv);
    cudaStream_t s = model->stream;
    m.jacobian_apply(dx.get(), t, cm, ca, dv.get(), dy.get(), s);
    dcgpu::cuda_check(cudaStreamSynchronize(s), "jacobian apply");
    std::vector<double> yb = dy.download(), yr;
    m.from_blocked(yb, yr);
    std::memcpy(y, yr.data(), m.ndof * sizeof(double));
    return DC_OK;
  });
}

int dc_pattern(const dc_model* model, int32_t* rowptr, size_t n_rowptr, int32_t* colidx, size_t n_colidx) {
  return guarded([&] {
    if (!model || !rowptr || !colidx) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    if (n_rowptr != m.rowptr.size() || n_colidx != m.colidx.size()) throw std::invalid_argument("size mismatch");
    std::memcpy(rowptr, m.rowptr.data(), n_rowptr * sizeof(int32_t));
    std::memcpy(colidx, m.colidx.data(), n_colidx * sizeof(int32_t));
    return DC_OK;
  });
}

int dc_dof_map(const dc_model* model, int64_t* ref_to_dev, size_t n) {
  return guarded([&] {
    if (!model || !ref_to_dev) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    if (static_cast<int64_t>(n) != m.ndof) throw std::invalid_argument("size mismatch");
    int64_t off = 0;
    for (size_t c = 0; c < m.comp_names.size(); ++c) {
      const int64_t nvc = static_cast<int64_t>(m.comp_vertices[c].size());
      for (int64_t k = 0; k < nvc; ++k)
        for (int s = 0; s < m.ns[c]; ++s) ref_to_dev[off + k * m.ns[c] + s] = (m.comp_node_offset[c] + k) * m.bs + s;
      off += nvc * m.ns[c];
    }
    return DC_OK;
  });
}

int dc_step_stage_newton(const dc_model* model, int32_t* counts, size_t n, size_t* n_out) {
  return guarded([&] {
    if (!model || !n_out) throw std::invalid_argument("null argument");
    const auto& v = model->solver->stats.step_stage_newton;
    *n_out = v.size();
    if (counts) {
      if (n < v.size()) throw std::invalid_argument("counts holds fewer entries than stage solves");
      for (size_t i = 0; i < v.size(); ++i) counts[i] = v[i];
    }
    return DC_OK;
  });
}

int dc_stats(const dc_model* model, int64_t* newton_iterations, int64_t* linear_iterations, int64_t* assemblies,
             int64_t* failed_steps) {
  return guarded([&] {
    if (!model) throw std::invalid_argument("null argument");
    const auto& st = model->solver->stats;
    if (newton_iterations) *newton_iterations = st.newton_iterations;
    if (linear_iterations) *linear_iterations = st.linear_iterations;
    if (assemblies) *assemblies = st.assemblies;
    if (failed_steps) *failed_steps = st.failed_steps;
    return DC_OK;
  });
}

int dc_expr_eval(const char* expression, const char* context_ini, const char* const* names, const double* values,
                 int32_t n, double* out) {
  return guarded([&] {
    if (!expression || !out || (n > 0 && (!names || !values))) throw std::invalid_argument("null argument");
    dcgpu::ParserContext ctx;
    if (context_ini) {
      dcgpu::Ini ini = dcgpu::Ini::parse(context_ini);
      if (ini.has_sub("parser_context")) ctx = dcgpu::ParserContext(ini.sub("parser_context"));
    }
    dcgpu::ProgramBuilder pb(ctx);
    dcgpu::Resolver res = [&](const std::string& nm) -> std::optional<dcgpu::Symbol> {
      for (int32_t i = 0; i < n; ++i)
        if (nm == names[i]) {
          dcgpu::Symbol s;
          s.is_input = true;
          s.input = static_cast<uint16_t>(i);
          return s;
        }
      if (nm == "no_value") {
        dcgpu::Symbol s;
        s.value = 1.7976931348623157e308;
        return s;
      }
      return std::nullopt;
    };
    pb.add_output(pb.compile_text(expression, res));
    dcgpu::Program p = pb.finish();
    std::vector<double> in(p.inputs.size());
    for (size_t i = 0; i < p.inputs.size(); ++i) in[i] = values[p.inputs[i]];
    *out = dcgpu::run_program_host(p, ctx, in.data());
    return DC_OK;
  });
}

int dc_server_create(int64_t budget_bytes, int32_t max_active, dc_server** out) {
  return dc_server_create_ex(budget_bytes, max_active, 0, out);
}

int dc_server_create_ex(int64_t budget_bytes, int32_t max_active, int32_t flags, dc_server** out) {
  return guarded([&] {
    if (!out) throw std::invalid_argument("null argument");
    *out = nullptr;
    if (flags & ~DC_SERVER_BATCH_KRYLOV) throw std::invalid_argument("unknown server flags");
    auto s = std::make_unique<dc_server>();
    s->server = std::make_unique<dcgpu::Server>(budget_bytes, max_active, (flags & DC_SERVER_BATCH_KRYLOV) != 0);
    *out = s.release();
    return DC_OK;
  });
}

int dc_server_batch_tuning(const dc_server* server, char* buf, size_t len) {
  return guarded([&] {
    if (!server || !buf || len == 0) throw std::invalid_argument("null argument");
    const std::string info = server->server->batch_tuning();
    std::strncpy(buf, info.c_str(), len - 1);
    buf[len - 1] = '\0';
    return DC_OK;
  });
}

int dc_server_batch_stats(const dc_server* server, dc_batch_stats* out) {
  return guarded([&] {
    if (!server || !out) throw std::invalid_argument("null argument");
    const dcgpu::BatchStats b = server->server->batch_stats();
    out->solves = b.solves;
    out->replays = b.replays;
    out->slot_replays = b.slot_replays;
    out->iterations = b.iterations;
    out->max_active = b.max_active;
    out->reserved = 0;
    out->replay_s = b.replay_s;
    out->wait_s = b.wait_s;
    return DC_OK;
  });
}

int dc_server_submit(dc_server* server, const char* ini_text, const char* overrides, const double* init_state,
                     size_t n_init, int64_t* request_id) {
  return guarded([&] {
    if (!server || !ini_text || !request_id) throw std::invalid_argument("null argument");
    std::vector<double> init;
    if (init_state && n_init) init.assign(init_state, init_state + n_init);
    *request_id = server->server->submit(ini_text, overrides ? overrides : "", std::move(init));
    return DC_OK;
  });
}

int dc_server_poll(dc_server* server, int32_t wait, dc_result* results, int32_t max, int32_t* n_out) {
  return guarded([&] {
    if (!server || !n_out || (max > 0 && !results)) throw std::invalid_argument("null argument");
    auto done = server->server->poll(wait != 0, max);
    for (size_t i = 0; i < done.size(); ++i) {
      const auto& r = done[i];
      dc_result& o = results[i];
      o.request_id = r.id;
      o.status = r.status;
      o.reserved = 0;
      o.queue_s = r.queue_s;
      o.run_s = r.run_s;
      o.latency_s = r.latency_s;
      o.n_dof = r.ndof;
      o.newton_iterations = r.newton_iterations;
      o.linear_iterations = r.linear_iterations;
      o.steps = r.steps;
      o.bytes_estimate = r.bytes_estimate;
      o.bytes_measured = r.bytes_measured;
      o.setup_s = r.setup_s;
      if (r.status != DC_OK && !r.error.empty()) g_last_error = r.error;
    }
    *n_out = static_cast<int32_t>(done.size());
    return DC_OK;
  });
}

int dc_server_take_state(dc_server* server, int64_t request_id, double* host_out, size_t n) {
  return guarded([&] {
    if (!server || !host_out) throw std::invalid_argument("null argument");
    std::vector<double> v;
    if (!server->server->take_state(request_id, v)) throw std::invalid_argument("no state for this request");
    if (v.size() != n) throw std::invalid_argument("size mismatch");
    std::memcpy(host_out, v.data(), n * sizeof(double));
    return DC_OK;
  });
}

int dc_server_estimate(const char* ini_text, const char* overrides, int64_t* bytes) {
  return guarded([&] {
    if (!ini_text || !bytes) throw std::invalid_argument("null argument");
    *bytes = dcgpu::Server::estimate_bytes(ini_text, overrides ? overrides : "");
    return DC_OK;
  });
}

int dc_server_destroy(dc_server* server) {
  return guarded([&] {
    delete server;
    return DC_OK;
  });
}

int dc_stream_handle(const dc_model* model, void** stream) {
  return guarded([&] {
    if (!model || !stream) throw std::invalid_argument("null argument");
    *stream = reinterpret_cast<void*>(model->stream);
    return DC_OK;
  });
}

int64_t dc_launch_count(void) { return dcgpu::launch_count(); }

int dc_selftest_barrier_timeout(double* gave_up_blocks, double* elapsed_ms) {
  return guarded([&] {
    if (!gave_up_blocks || !elapsed_ms) throw std::invalid_argument("null argument");
    if (dcgpu::barrier_selftest(gave_up_blocks, elapsed_ms) != 0)
      throw std::runtime_error("barrier self-test: CUDA error");
    return DC_OK;
  });
}

namespace {

void require_device() {
  int dev_count = 0;
  dcgpu::cuda_check(cudaGetDeviceCount(&dev_count), "cudaGetDeviceCount");
  if (dev_count == 0) throw dcgpu::CudaError("no CUDA device");
}

// host CSR graph -> device copies (validated)
struct HostGraph {
  dcgpu::DeviceBuffer<int32_t> rowptr, colidx, group;
  HostGraph(int64_t n, const int32_t* rp, const int32_t* ci, const int32_t* grp) {
    if (n <= 0 || n >= (int64_t(1) << 31) || !rp || !ci) throw std::invalid_argument("bad graph");
    std::vector<int32_t> r(rp, rp + n + 1);
    if (r[0] != 0) throw std::invalid_argument("rowptr[0] must be 0");
    for (int64_t i = 0; i < n; ++i)
      if (r[i + 1] < r[i]) throw std::invalid_argument("rowptr must not decrease");
    std::vector<int32_t> c(ci, ci + r[n]);
    for (int32_t v : c)
      if (v < 0 || v >= n) throw std::invalid_argument("column index out of range");
    rowptr.upload(r);
    colidx.upload(c);
    if (grp) group.upload(std::vector<int32_t>(grp, grp + n));
  }
};

double param(const std::string& params, const std::string& key, double dflt) {
  size_t pos = 0;
  while (pos < params.size()) {
    size_t end = params.find(';', pos);
    if (end == std::string::npos) end = params.size();
    const std::string item = params.substr(pos, end - pos);
    const size_t eq = item.find('=');
    if (eq != std::string::npos && item.substr(0, eq) == key) return std::stod(item.substr(eq + 1));
    pos = end + 1;
  }
  return dflt;
}

}  // namespace

int dc_selftest_color(int64_t nrows, const int32_t* rowptr, const int32_t* colidx, int32_t* colour_out,
                      int32_t* ncolours) {
  return guarded([&] {
    if (!colour_out || !ncolours) throw std::invalid_argument("null argument");
    require_device();
    HostGraph g(nrows, rowptr, colidx, nullptr);
    dcgpu::DeviceGraph dg;
    dg.n = nrows;
    dg.rowptr = g.rowptr.get();
    dg.colidx = g.colidx.get();
    dcgpu::DeviceBuffer<int32_t> colour(static_cast<size_t>(nrows));
    *ncolours = dcgpu::color_rows(dg, colour.get(), cudaStreamLegacy);
    dcgpu::cuda_check(cudaMemcpy(colour_out, colour.get(), nrows * sizeof(int32_t), cudaMemcpyDeviceToHost), "colour");
    return DC_OK;
  });
}

int dc_selftest_aggregate(int64_t nrows, const int32_t* rowptr, const int32_t* colidx, const int32_t* group,
                          int32_t distance, int32_t* agg_out, int64_t* naggregates) {
  return guarded([&] {
    if (!agg_out || !naggregates) throw std::invalid_argument("null argument");
    if (distance != 1 && distance != 2) throw std::invalid_argument("distance must be 1 or 2");
    require_device();
    HostGraph g(nrows, rowptr, colidx, group);
    dcgpu::DeviceGraph dg;
    dg.n = nrows;
    dg.rowptr = g.rowptr.get();
    dg.colidx = g.colidx.get();
    dg.group = group ? g.group.get() : nullptr;
    dcgpu::DeviceBuffer<int32_t> agg(static_cast<size_t>(nrows));
    *naggregates = dcgpu::aggregate_mis(dg, distance, agg.get(), cudaStreamLegacy);
    dcgpu::cuda_check(cudaMemcpy(agg_out, agg.get(), nrows * sizeof(int32_t), cudaMemcpyDeviceToHost), "aggregate");
    return DC_OK;
  });
}

int dc_selftest_precond(const char* kind, const char* params, int64_t nrows, int32_t bs, const int32_t* rowptr,
                        const int32_t* colidx, const double* vals, const int32_t* group, const double* r, double* z,
                        int32_t fp32, double* info) {
  return guarded([&] {
    if (!kind || !vals || !r || !z) throw std::invalid_argument("null argument");
    if (bs < 1 || bs > 8) throw std::invalid_argument("block size must be in [1, 8]");
    require_device();
    const std::string k = kind, prm = params ? params : "";
    HostGraph g(nrows, rowptr, colidx, group);
    const int64_t nnzb = rowptr[nrows];
    std::vector<int32_t> diag(static_cast<size_t>(nrows), -1);
    for (int64_t i = 0; i < nrows; ++i)
      for (int32_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
        if (colidx[e] == i) diag[i] = e;
    for (int32_t d : diag)
      if (d < 0) throw std::invalid_argument("a row without its diagonal block");
    const size_t b2 = static_cast<size_t>(bs) * bs, nv = static_cast<size_t>(nrows) * bs;
    dcgpu::DeviceBuffer<int32_t> ddiag, status(1);
    ddiag.upload(diag);
    dcgpu::DeviceBuffer<double> dval, dinv(static_cast<size_t>(nrows) * b2), dr, dz(nv);
    dval.upload(std::vector<double>(vals, vals + nnzb * b2));
    dr.upload(std::vector<double>(r, r + nv));
    dcgpu::DeviceBuffer<float> fval(static_cast<size_t>(nnzb) * b2), fdinv(static_cast<size_t>(nrows) * b2),
        fr(nv), fz(nv);
    cudaStream_t s = cudaStreamLegacy;
    dcgpu::cuda_check(cudaMemset(status.get(), 0, sizeof(int)), "memset");
    dcgpu::Bsr A;
    A.nrows = static_cast<int>(nrows);
    A.bs = bs;
    A.nnzb = nnzb;
    A.rowptr = g.rowptr.get();
    A.colidx = g.colidx.get();
    A.val = dval.get();
    dcgpu::block_jacobi_setup(A, ddiag.get(), dinv.get(), status.get(), s, fdinv.get());
    dcgpu::to_float(static_cast<int64_t>(nnzb * b2), dval.get(), fval.get(), s);
    dcgpu::to_float(static_cast<int64_t>(nv), dr.get(), fr.get(), s);
    std::unique_ptr<dcgpu::Preconditioner> pc;
    double inf[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (k == "AMG") {
      auto amg = std::make_unique<dcgpu::Amg>();
      const int smi = static_cast<int>(param(prm, "smoother", 0));
      amg->smoother = smi == 0   ? dcgpu::Amg::Smoother::Jacobi
                      : smi == 1 ? dcgpu::Amg::Smoother::L1Jacobi
                      : smi == 2 ? dcgpu::Amg::Smoother::GaussSeidel
                                 : dcgpu::Amg::Smoother::Ilu0;
      amg->omega = param(prm, "relaxation", smi == 0 ? 0.85 : 1.0);
      amg->coarse_sweeps = static_cast<int>(param(prm, "coarse_sweeps", 6));
      amg->max_levels = static_cast<int>(param(prm, "max_level", 10));
      amg->coarsen_target = static_cast<int64_t>(param(prm, "coarsen_target", 0));
      amg->mis_distance = static_cast<int>(param(prm, "aggregation_distance", 2));
      amg->correction = param(prm, "coarse_correction", 1.0);
      amg->finest_post_smoothing = param(prm, "finest_post_smoothing", 1.0) != 0.0;
      amg->w_levels = static_cast<int>(param(prm, "w_levels", 0));
      amg->warp_rows_below = static_cast<int64_t>(param(prm, "warp_rows_below", dcgpu::Amg::kWarpRowsBelow));
      amg->build(nrows, bs, nnzb, g.rowptr.get(), g.colidx.get(), ddiag.get(), group ? g.group.get() : nullptr, s);
      amg->setup(dval.get(), dinv.get(), fdinv.get(), fp32 != 0, status.get(), s);
      inf[0] = amg->levels();
      inf[1] = amg->dense_coarse() ? static_cast<double>(amg->rows(amg->levels() - 1) * bs) : 0.0;
      for (int l = 0; l < amg->levels() && l < 6; ++l) inf[2 + l] = static_cast<double>(amg->rows(l));
      pc = std::move(amg);
    } else {
      dcgpu::ColorPrecond::Kind kd;
      if (k == "SSOR") kd = dcgpu::ColorPrecond::Kind::Ssor;
      else if (k == "SOR") kd = dcgpu::ColorPrecond::Kind::Sor;
      else if (k == "ILU") kd = dcgpu::ColorPrecond::Kind::Ilu0;
      else if (k == "DILU") kd = dcgpu::ColorPrecond::Kind::Dilu;
      else throw std::invalid_argument("unknown preconditioner kind " + k);
      auto mc = std::make_unique<dcgpu::ColorPrecond>();
      mc->omega = param(prm, "relaxation", 1.0);
      mc->iterations = static_cast<int>(param(prm, "iterations", 1));
      mc->build(kd, nrows, bs, nnzb, g.rowptr.get(), g.colidx.get(), ddiag.get(), s);
      mc->setup(dval.get(), dinv.get(), fdinv.get(), fp32 != 0, status.get(), s);
      inf[0] = mc->colors();
      pc = std::move(mc);
    }
    int st = 0;
    dcgpu::cuda_check(cudaMemcpy(&st, status.get(), sizeof(int), cudaMemcpyDeviceToHost), "status");
    if (st) throw dcgpu::StepFailure("singular block in the preconditioner set-up");
    std::vector<double> out(nv);
    if (fp32) {
      pc->apply(fr.get(), fz.get(), nullptr, 0, s);
      std::vector<float> o(nv);
      dcgpu::cuda_check(cudaMemcpy(o.data(), fz.get(), nv * sizeof(float), cudaMemcpyDeviceToHost), "result");
      for (size_t q = 0; q < nv; ++q) out[q] = o[q];
    } else {
      pc->apply(dr.get(), dz.get(), nullptr, 0, s);
      dcgpu::cuda_check(cudaMemcpy(out.data(), dz.get(), nv * sizeof(double), cudaMemcpyDeviceToHost), "result");
    }
    std::memcpy(z, out.data(), nv * sizeof(double));
    if (info) std::memcpy(info, inf, sizeof(inf));
    return DC_OK;
  });
}

int dc_precond_info(const dc_model* model, char* buf, size_t len) {
  return guarded([&] {
    if (!model || !buf || len == 0) throw std::invalid_argument("null argument");
    const std::string info = model->solver->precond_info();
    std::strncpy(buf, info.c_str(), len - 1);
    buf[len - 1] = '\0';
    return DC_OK;
  });
}

int dc_model_jit_status(const dc_model* model, char* buf, size_t len) {
  return guarded([&] {
    if (!model || !buf || len == 0) throw std::invalid_argument("null argument");
    std::strncpy(buf, model->model->jit_status.c_str(), len - 1);
    buf[len - 1] = '\0';
    return DC_OK;
  });
}

int dc_selftest_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  return guarded([&] {
    if (!fp64_tflops || !fp32_tflops) throw std::invalid_argument("null argument");
    int dev_count = 0;
    dcgpu::cuda_check(cudaGetDeviceCount(&dev_count), "cudaGetDeviceCount");
    if (dev_count == 0) throw dcgpu::CudaError("no CUDA device");
    if (dcgpu::fma_peaks(fp64_tflops, fp32_tflops) != 0) throw dcgpu::CudaError("FMA throughput probe failed");
    return DC_OK;
  });
}

int dc_profile_enable(dc_model* model, int enabled) {
  return guarded([&] {
    if (!model) throw std::invalid_argument("null argument");
    model->solver->enable_profiling(enabled != 0);
    return DC_OK;
  });
}

int dc_profile_get(const dc_model* model, double* ms, int64_t* calls, int32_t n_categories) {
  return guarded([&] {
    if (!model || !ms || !calls) throw std::invalid_argument("null argument");
    const auto& kt = model->solver->kernel_times;
    for (int32_t c = 0; c < n_categories; ++c) {
      const bool ok = c < dcgpu::Solver::kTimerCategories;
      ms[c] = ok ? kt.ms[c] : 0.0;
      calls[c] = ok ? kt.calls[c] : 0;
    }
    return DC_OK;
  });
}

int dc_reduce(const dc_model* model, const char* reduce_ini, dc_reduce_value* out, size_t n, size_t* n_out) {
  return guarded([&] {
    if (!model || !n_out) throw std::invalid_argument("null argument");
    const auto& m = *model->model;
    dcgpu::Ini sec;
    if (reduce_ini) {
      dcgpu::Ini t = dcgpu::Ini::parse(reduce_ini);
      sec = t.has_sub("model.reduce") ? t.sub("model.reduce") : t;
    } else {
      sec = m.cfg.sub("model").sub("reduce");
    }
    *n_out = sec.sub_keys().size();
    if (!out) return DC_OK;
    if (n < *n_out) throw std::invalid_argument("output array too small");
    auto res = m.reduce(model->solver->state_device(), model->solver->time(), sec, model->stream);
    for (size_t k = 0; k < res.size(); ++k) {
      std::memset(out[k].key, 0, sizeof(out[k].key));
      std::strncpy(out[k].key, res[k].key.c_str(), sizeof(out[k].key) - 1);
      out[k].value = res[k].value;
      out[k].error = res[k].error ? 1 : 0;
      out[k].warn = res[k].warn ? 1 : 0;
    }
    return DC_OK;
  });
}

int dc_spmv_format(const dc_model* model, int32_t* format, double* bsr_us, double* sell_us) {
  return guarded([&] {
    if (!model || !format) throw std::invalid_argument("null argument");
    const auto& s = *model->solver;
    *format = s.spmv_format;
    if (bsr_us) *bsr_us = s.spmv_tune_us[0];
    if (sell_us) *sell_us = s.spmv_tune_us[1];
    return DC_OK;
  });
}

int dc_set_mixed_precision(dc_model* model, int enabled) {
  return guarded([&] {
    if (!model) throw std::invalid_argument("null argument");
    model->solver->enable_mixed(enabled != 0);
    return DC_OK;
  });
}

}  // extern "C"
