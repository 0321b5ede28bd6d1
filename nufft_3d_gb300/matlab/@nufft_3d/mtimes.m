% y = obj * x: fNUFT(x), or aNUFT(x) for the object returned by obj'.
% (No counterpart in the reference class, which has no mtimes; it lets
% solvers use the object as a linear operator.)
function y = mtimes(obj, x)
if ~isa(obj, 'nufft_3d')
    error('nufft_3d must be the left operand of *');
end
if obj.adjoint
    y = obj.aNUFT(x);
else
    y = obj.fNUFT(x);
end
