"""TimeControl: the reference's time-step bookkeeping (utilities.cc:31-95)."""
import math


def _round(x):
    """std::round: halves away from zero."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


class TimeControl:
    def setup(self, final_time, tick_time, time_step, max_time_step=0):
        self.final_time = final_time
        self.time = 0.0
        self.tick_size = tick_time
        self.time_step_number = 0
        # rounded so that the step divides the interval (utilities.cc:38)
        n = max(_round((final_time - self.time) / time_step), 1.0)
        self.time_step = (final_time - self.time) / n
        self.max_time_step = _round((final_time - self.time) / self.time_step) if max_time_step == 0 \
            else max_time_step

    def set_time_step(self, dt):
        self.time_step = dt

    def advance_time_step(self):
        self.time_step_number += 1
        self.time += self.time_step

    def done(self):
        return self.time >= self.final_time or self.time_step_number > self.max_time_step

    def at_tick(self):
        return int(self.time / self.tick_size) != int((self.time - self.time_step) / self.tick_size)
