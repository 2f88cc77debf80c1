-- Sod tube with the limiter set only through slopeLimiterName: the solver reads
-- slopeLimiter, so Superbee stays in force
solverName = 'EulerRoe'
slopeLimiterName = 'MinMod'
integratorName = 'ForwardEuler'
size = {1024}
xmin = {0}
xmax = {1}
boundaryMethods = {{min = 'FREEFLOW', max = 'FREEFLOW'}}
cfl = 0.5
