/*
 * mkg_pacing.h -- event-based pacing and the reference's step schedule.
 *
 * Pacer follows the semantics of myokit's ESys event system
 * (myokit/_sim/pacing.h:168-600): an event queue ordered by start time,
 * periodic events rescheduled after they fire, a multiplier counting
 * remaining repeats, and float-tolerant time comparisons (pacing.h:69-80).
 *
 * Schedule follows the step-size logic of sim_step (openclsim.c:1051-1162):
 * a fixed step grid tmin + i*dt, shortened ("intermediary" steps that do not
 * advance i) to land exactly on tmax, on the next pacing event and on the
 * next log time. Host-only C++; used by mkg_host.cu and by the CPU test hook
 * mkg_schedule_preview.
 */
#ifndef MKG_PACING_H
#define MKG_PACING_H

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

namespace mkg {

enum PacerStatus {
    PACER_OK = 0,
    PACER_NON_ZERO_MULTIPLIER = -23,   /* pacing.h:60 */
    PACER_NEGATIVE_PERIOD = -24,
    PACER_NEGATIVE_MULTIPLIER = -25,
    PACER_NEGATIVE_TIME_INCREMENT = -40,
    PACER_SIMULTANEOUS_EVENT = -50,
};

/* |a - b| within relative DBL_EPSILON (pacing.h:74) */
inline bool time_eq(double a, double b)
{
    if (a == b) return true;
    const double s = std::fabs(a) > std::fabs(b) ? std::fabs(a) : std::fabs(b);
    return std::fabs(a - b) / s < DBL_EPSILON;
}

/* a >= b, or equal within tolerance (pacing.h:80) */
inline bool time_geq(double a, double b) { return a >= b || time_eq(a, b); }

class Pacer {
public:
    struct Event {
        double level, duration, start, period, multiplier;
        int next;   /* index of the next queued event, or -1 */
    };

    /* rows of (level, start, duration, period, multiplier) */
    int populate(const double *rows, int64_t n)
    {
        events_.clear();
        for (int64_t i = 0; i < n; ++i) {
            Event e;
            e.level = rows[5 * i + 0];
            e.start = rows[5 * i + 1];
            e.duration = rows[5 * i + 2];
            e.period = rows[5 * i + 3];
            e.multiplier = rows[5 * i + 4];
            e.next = -1;
            if (e.period == 0 && e.multiplier != 0)
                return PACER_NON_ZERO_MULTIPLIER;
            if (e.period < 0) return PACER_NEGATIVE_PERIOD;
            if (e.multiplier < 0) return PACER_NEGATIVE_MULTIPLIER;
            events_.push_back(e);
        }
        original_ = events_;
        return PACER_OK;
    }

    /* Restores the populated events and sets the time to t0. */
    int reset(double t0)
    {
        events_ = original_;
        head_ = -1;
        fire_ = -1;
        for (int i = 0; i < (int)events_.size(); ++i) {
            int st = PACER_OK;
            head_ = schedule(head_, i, &st);
            if (st != PACER_OK) return st;
        }
        time_ = t0;
        tnext_ = t0;
        tdown_ = t0;
        level_ = 0;
        return PACER_OK;
    }

    /* Advances to new_time, firing and retiring events (pacing.h:483-548). */
    int advance(double new_time)
    {
        if (new_time < time_) return PACER_NEGATIVE_TIME_INCREMENT;
        time_ = new_time;
        while (time_geq(time_, tnext_)) {
            if (fire_ >= 0 && time_geq(tnext_, tdown_)) {
                fire_ = -1;
                level_ = 0;
            }
            if (head_ >= 0 && time_geq(tnext_, events_[head_].start)) {
                fire_ = head_;
                Event &f = events_[fire_];
                head_ = f.next;
                tdown_ = f.start + f.duration;
                level_ = f.level;
                if (f.period > 0) {
                    if (f.multiplier != 1) {
                        if (f.multiplier > 1) f.multiplier -= 1;
                        f.start += f.period;
                        int st = PACER_OK;
                        head_ = schedule(head_, fire_, &st);
                        if (st != PACER_OK) return st;
                    } else {
                        f.period = 0;
                    }
                }
                if (head_ >= 0 && time_eq(events_[head_].start, tdown_))
                    tdown_ = events_[head_].start;
            }
            tnext_ = HUGE_VAL;
            if (fire_ >= 0 && tnext_ > tdown_) tnext_ = tdown_;
            if (head_ >= 0 && tnext_ > events_[head_].start)
                tnext_ = events_[head_].start;
        }
        return PACER_OK;
    }

    double next_time() const { return tnext_; }
    double level() const { return level_; }

private:
    /* Inserts event i after every queued event that starts no later than it
     * (pacing.h:192-212); equal start times are an error. */
    int schedule(int head, int i, int *status)
    {
        *status = PACER_OK;
        events_[i].next = -1;
        if (head < 0) return i;
        if (events_[i].start < events_[head].start) {
            events_[i].next = head;
            return i;
        }
        int e = head;
        while (events_[e].next >= 0 &&
               events_[i].start >= events_[events_[e].next].start)
            e = events_[e].next;
        if (events_[i].start == events_[e].start)
            *status = PACER_SIMULTANEOUS_EVENT;
        events_[i].next = events_[e].next;
        events_[e].next = i;
        return head;
    }

    std::vector<Event> events_, original_;
    int head_ = -1, fire_ = -1;
    double time_ = 0, tnext_ = 0, tdown_ = 0, level_ = 0;
};

/* One scheduled step as seen by the host. */
struct StepRecord {
    double t, dt, pace, t_end;
    bool log;
};

/* The reference's step loop state (openclsim.c:1036-1162). */
class Schedule {
public:
    int begin(const Pacer &proto, double tmin, double tmax, double dt,
              double log_interval)
    {
        pacer_ = proto;
        tmin_ = tmin;
        tmax_ = tmax;
        default_dt_ = dt;
        log_interval_ = log_interval;
        int st = pacer_.reset(tmin);
        if (st != PACER_OK) return st;
        st = pacer_.advance(tmin);
        if (st != PACER_OK) return st;
        tnext_pace_ = pacer_.next_time();
        pace_ = pacer_.level();
        time_ = tmin;
        istep_ = 1;
        inext_log_ = 0;
        tnext_log_ = tmin;
        done_ = !(tmin < tmax);
        return PACER_OK;
    }

    bool done() const { return done_; }
    double time() const { return time_; }

    /* Produces the next step; sets done() once time reaches tmax. */
    int next(StepRecord *r)
    {
        const bool logging = time_ >= tnext_log_;
        bool intermediary = false;
        double dt = tmin_ + (double)istep_ * default_dt_ - time_;
        double d = tmax_ - time_;
        if (d > 0 && d < dt) { dt = d; intermediary = true; }
        d = tnext_pace_ - time_;
        if (d > 0 && d < dt) { dt = d; intermediary = true; }
        d = tnext_log_ - time_;
        if (d > 0 && d < dt) { dt = d; intermediary = true; }
        if (!intermediary) istep_++;
        r->t = time_;
        r->dt = dt;
        r->pace = pace_;
        r->log = logging;
        if (logging) {
            inext_log_++;
            tnext_log_ = tmin_ + (double)inext_log_ * log_interval_;
        }
        time_ += dt;
        r->t_end = time_;
        const int st = pacer_.advance(time_);
        if (st != PACER_OK) return st;
        tnext_pace_ = pacer_.next_time();
        pace_ = pacer_.level();
        if (time_ >= tmax_) done_ = true;
        return PACER_OK;
    }

    /* Would the next step write a log row? */
    bool next_logs() const { return time_ >= tnext_log_; }

private:
    Pacer pacer_;
    double tmin_ = 0, tmax_ = 0, default_dt_ = 0, log_interval_ = 1;
    double time_ = 0, tnext_pace_ = 0, pace_ = 0, tnext_log_ = 0;
    uint64_t istep_ = 1, inext_log_ = 0;
    bool done_ = true;
};

}  // namespace mkg

#endif /* MKG_PACING_H */
