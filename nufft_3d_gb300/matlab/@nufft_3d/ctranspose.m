% t = obj': the same transform with fNUFT and aNUFT exchanged under *
% (t * k = obj.aNUFT(k)).  t shares obj's plan and keeps obj alive; deleting
% t leaves the plan to obj.  (No counterpart in the reference class.)
function t = ctranspose(obj)
t = nufft_3d();
t.J = obj.J; t.u = obj.u; t.N = obj.N; t.alpha = obj.alpha; t.radial = obj.radial;
t.gpu = obj.gpu; t.K = obj.K; t.U = obj.U; t.d = obj.d; t.nnz = obj.nnz;
t.plan = obj.plan;
t.M = obj.M;
t.adjoint = ~obj.adjoint;
t.owner = obj;
end
