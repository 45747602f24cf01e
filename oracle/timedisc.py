"""Restatement of FLEXI's time loop control -- TEST INFRASTRUCTURE ONLY (the checker of fg_run's UpdateTimeStep).

Follows src/timedisc/timedisc.f90:TimeDisc (:95-212: tAnalyze = MIN(t+analyze_dt, tEnd), the loop
UpdateTimeStep -> CalcForcing -> TimeStep -> t += dt -> AnalyzeTimeStep, EXIT on doFinalize),
src/timedisc/timedisc_func.f90:UpdateTimeStep (:215-268), EvalTimeStep (:433-454), AnalyzeTimeStep (:273-385:
maxIter, tAnalyze = MIN(tAnalyze+analyze_dt, tEnd)) and src/analyze/analyze.f90:124-130 (analyze_dt <= 0 means
tEnd). The time step comes from a callback (the oracle's CALCTIMESTEP), the step from another (the oracle's
TimeStepByLSERKW2), so the control logic is checked on its own and drives the CPU restatement of the solver.
"""
import math

EPS = 2.220446049250313e-16  # EPSILON(0.) of the reference's default 8-byte REAL


class KillTimestep(RuntimeError):
    """EvalTimeStep's Abort: 'Critical Kill timestep reached'."""


class TimeDiscLoop:
    def __init__(self, calc_timestep, timestep, t=0.0, tEnd=math.inf, analyze_dt=0.0, dtmin=-1.0, dtkill=-1.0, nCalcTimeStepMax=1,
                 maxIter=-1):
        self.calc_timestep, self.timestep = calc_timestep, timestep
        self.tEnd = tEnd
        self.analyze_dt = analyze_dt if analyze_dt > 0.0 else tEnd  # analyze.f90:127-130
        self.dtmin, self.dtkill, self.nCalcMax, self.maxIter = dtmin, dtkill, nCalcTimeStepMax, maxIter
        self.t = t
        self.tAnalyze = min(t + self.analyze_dt, tEnd)  # timedisc.f90:107
        self.nCalcTimeStep = 0  # timedisc.f90:111
        self.dt_minOld = -999.0  # timedisc_func.f90:195
        self.dt = 0.0
        self.dt_min_calc = 0.0
        self.iter = 0
        self.nDtLimited = 0
        self.doAnalyze = self.doFinalize = False
        self.analyze_times = []  # times at which AnalyzeTimeStep analysed (doAnalyze)

    def eval_timestep(self):
        """EvalTimeStep (timedisc_func.f90:433-454)."""
        dt, err = self.calc_timestep()
        if err != 0:
            raise RuntimeError(f"CALCTIMESTEP errType {err}")
        if dt < self.dtmin:
            dt = self.dtmin
            self.nDtLimited += 1
        if dt < self.dtkill:
            raise KillTimestep(f"critical kill time step reached at t={self.t}")
        return dt

    def update_timestep(self):
        """UpdateTimeStep (timedisc_func.f90:215-268)."""
        if self.nCalcTimeStep >= 1:
            self.nCalcTimeStep -= 1
            return
        d_min = self.eval_timestep()
        self.dt_min_calc = d_min
        d_ana = self.tAnalyze - self.t
        d_end = self.tEnd - self.t
        dt = min(d_min, d_ana, d_end)
        if dt == d_ana:
            self.doAnalyze = True
        if dt == d_end:
            self.doAnalyze = self.doFinalize = True
        dt = min(x for x in (d_min, d_ana, d_end) if x > 0.0)
        q = abs(self.dt_minOld / dt - 1.0) ** 2 * 100.0 + EPS
        self.nCalcTimeStep = min(math.floor(abs(math.log10(q))), self.nCalcMax) - 1
        self.dt_minOld = dt
        if d_ana - dt < dt / 100.0 and d_ana > 0.0:
            dt = d_ana
            self.doAnalyze = True
        if d_end - dt < dt / 100.0 and d_end > 0.0:
            dt = d_end
            self.doAnalyze = self.doFinalize = True
        self.dt = dt

    def step(self):
        """One pass of the TimeDisc loop (timedisc.f90:190-212) with the time bookkeeping of AnalyzeTimeStep.
        Returns True when the loop would EXIT (doFinalize)."""
        self.update_timestep()
        self.timestep(self.t, self.dt)
        self.iter += 1
        self.t = self.t + self.dt
        if self.iter == self.maxIter:  # timedisc_func.f90:316-319
            self.tEnd = self.tAnalyze = self.t
            self.doAnalyze = self.doFinalize = True
        if self.doAnalyze:
            self.analyze_times.append(self.t)
            self.tAnalyze = min(self.tAnalyze + self.analyze_dt, self.tEnd)
            self.doAnalyze = False
        return self.doFinalize

    def run(self, max_steps):
        """Steps until doFinalize or max_steps passes."""
        for _ in range(max_steps):
            if self.doFinalize:
                break
            self.step()
        return self.t
