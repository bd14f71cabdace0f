// nbg_batch_async.cu -- the asynchronous batch (nbg_batch_create / submit /
// run / wait / destroy in include/nbg.h): nbg_batch_integrate_transits run
// on a library host thread, so that the caller's thread is free meanwhile.
// Host code only; the GPU work is the batched entry point's own.
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nbg.h"
#include "nbg_internal.cuh"

using namespace nbg;

namespace {

enum BatchState { BATCH_IDLE = 0, BATCH_RUNNING = 1, BATCH_FINISHED = 2 };

struct Arrays {
  double *t, *x, *v;
  const double* m;
  double *xerror, *verror, *jac_step, *jac_error, *dqdt;
  const uint8_t* pair;
  const double* jac_init;
  double *tt, *dtdq0, *dtdelements;
  int64_t* count;
  uint32_t* status;
};

}  // namespace

struct nbg_batch {
  nbg_context* ctx = nullptr;
  std::vector<nbg_system_desc> desc;
  Arrays a{};
  bool submitted = false;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  int state = BATCH_IDLE;  // under mu
  int rc = NBG_OK;         // the finished run's result (under mu)
  std::string msg;         // its error message (under mu)
};

namespace {

void run_worker(nbg_batch* b) {
  const Arrays& a = b->a;
  const int rc = nbg_batch_integrate_transits(b->ctx, (int)b->desc.size(), b->desc.data(), a.t, a.x, a.v, a.m,
                                              a.xerror, a.verror, a.jac_step, a.jac_error, a.dqdt, a.pair,
                                              a.jac_init, a.tt, a.dtdq0, a.dtdelements, a.count, a.status);
  char buf[1024];
  buf[0] = '\0';
  if (rc) nbg_last_error(buf, sizeof(buf));  // the message is this thread's; hand it to the waiter
  std::lock_guard<std::mutex> lk(b->mu);
  b->rc = rc;
  b->msg = buf;
  b->state = BATCH_FINISHED;
  b->cv.notify_all();
}

}  // namespace

extern "C" {

int nbg_batch_create(nbg_context* ctx, int nsys, const nbg_system_desc* desc, nbg_batch** out) {
  if (!out) return set_error(NBG_EINVAL, "out is NULL");
  *out = nullptr;
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !desc) return set_error(NBG_EINVAL, "nsys = %d", nsys);
  for (int s = 0; s < nsys; s++) {
    const nbg_system_desc& d = desc[s];
    if (d.n < NBG_MIN_BODIES || d.n > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside the built range %d..%d", s, d.n, NBG_MIN_BODIES,
                       NBG_MAX_BODIES);
    if (d.ti < 0 || d.ti >= d.n) return set_error(NBG_EINVAL, "system %d: ti = %d not in 0..%d", s, d.ti, d.n - 1);
    if (d.ntt < 1) return set_error(NBG_EINVAL, "system %d: ntt = %d < 1", s, d.ntt);
    if (!(d.h != 0.0) || !std::isfinite(d.h) || !std::isfinite(d.tmax))
      return set_error(NBG_EINVAL, "system %d: h = %g, tmax = %g", s, d.h, d.tmax);
  }
  nbg_batch* b = new nbg_batch();
  b->ctx = ctx;
  b->desc.assign(desc, desc + nsys);
  *out = b;
  return NBG_OK;
}

int nbg_batch_submit(nbg_batch* b, double* t, double* x, double* v, const double* m, double* xerror, double* verror,
                     double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair, const double* jac_init,
                     double* tt, double* dtdq0, double* dtdelements, int64_t* count, uint32_t* status) {
  if (!b) return set_error(NBG_EINVAL, "batch is NULL");
  if (!t || !x || !v || !m || !xerror || !verror || !jac_step || !jac_error || !dqdt || !pair || !jac_init || !tt ||
      !dtdq0 || !dtdelements || !count)
    return set_error(NBG_EINVAL, "NULL array argument");
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->state != BATCH_IDLE)
    return set_error(NBG_EINVAL, "the batch is running or its result has not been collected (nbg_batch_wait)");
  b->a = Arrays{t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair, jac_init, tt, dtdq0, dtdelements, count,
                status};
  b->submitted = true;
  return NBG_OK;
}

int nbg_batch_run(nbg_batch* b) {
  if (!b) return set_error(NBG_EINVAL, "batch is NULL");
  std::lock_guard<std::mutex> lk(b->mu);
  if (!b->submitted) return set_error(NBG_EINVAL, "no arrays submitted (nbg_batch_submit)");
  if (b->state != BATCH_IDLE)
    return set_error(NBG_EINVAL, "the batch is running or its result has not been collected (nbg_batch_wait)");
  if (b->worker.joinable()) b->worker.join();  // the previous run's thread, already finished
  b->state = BATCH_RUNNING;
  b->rc = NBG_OK;
  b->msg.clear();
  try {
    b->worker = std::thread(run_worker, b);
  } catch (...) {
    b->state = BATCH_IDLE;
    return set_error(NBG_ENOMEM, "could not start the batch's host thread");
  }
  return NBG_OK;
}

int nbg_batch_wait(nbg_batch* b, int32_t timeout_ms) {
  if (!b) return set_error(NBG_EINVAL, "batch is NULL");
  int rc;
  std::string msg;
  {
    std::unique_lock<std::mutex> lk(b->mu);
    if (b->state == BATCH_IDLE) return set_error(NBG_EINVAL, "the batch is not running (nbg_batch_run)");
    auto done = [&] { return b->state == BATCH_FINISHED; };
    if (timeout_ms < 0) b->cv.wait(lk, done);
    else if (!b->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
      return set_error(NBG_ETIMEOUT, "the batch is still running after %d ms", timeout_ms);
    rc = b->rc;
    msg = b->msg;
    b->state = BATCH_IDLE;
    // the worker's last use of the lock is over; joining under it keeps the
    // thread object away from a concurrent nbg_batch_run
    if (b->worker.joinable()) b->worker.join();
  }
  if (rc) return set_error(rc, "%s", msg.c_str());
  return NBG_OK;
}

int nbg_batch_destroy(nbg_batch* b) {
  if (!b) return NBG_OK;
  if (b->worker.joinable()) b->worker.join();  // a started run ends before its arrays are released
  delete b;
  return NBG_OK;
}

}  // extern "C"
