% im = obj.iNUFT(raw, maxit, damp, W, solver, tol): iterative reconstruction.
%
%  raw   complex [M nc] or [nr ny nc]
%  maxit iterations (0 or 1: regridding aNUFT(d .* raw)); default 20
%  damp  Tikhonov damping; default 0
%  W     [] or a scalar, [ny] or [nr*ny] nonnegative weights (times d)
%  solver 'minres' (default, as the reference) or 'cg'; tol default 1e-4
%
% Each coil is solved as its own system (A'WA + damp^2 I) x = A'W raw on the
% GPU (iNUFT.m:2-138, 224-227 of the reference, default path).  The
% experimental constraints of the reference are not implemented.
function [im, iters] = iNUFT(obj, raw, maxit, damp, W, solver, tol)
if nargin < 3 || isempty(maxit), maxit = 20; end
if nargin < 4 || isempty(damp), damp = 0; end
if nargin < 5, W = []; end
if nargin < 6 || isempty(solver), solver = 'minres'; end
if nargin < 7 || isempty(tol), tol = 1e-4; end
validateattributes(maxit, {'numeric'}, {'scalar', 'finite', 'integer', 'nonnegative'}, '', 'maxit');
validateattributes(damp, {'numeric'}, {'scalar', 'finite', 'nonnegative'}, '', 'damp');
[nc, nr, ny] = obj.raw_shape(raw);
Wv = [];
if numel(W) > 1
    W = double(W(:));
    if numel(W) ~= obj.M
        if isempty(ny), ny = numel(W); nr = obj.M / ny; end
        if mod(nr, 1) || nr * ny ~= obj.M
            error('W must be a vector of length ny or ny*nr');
        end
        W = repmat(reshape(W, 1, ny), nr, 1);
    end
    if any(~isfinite(W(:))) || any(W(:) < 0)
        error('W must be finite and nonnegative');
    end
    Wv = single(W(:));
end
raw = single(reshape(raw, obj.M, nc));
if isreal(raw), raw = complex(raw); end
[im, iters] = nufft3d_mex('inverse', obj.plan, raw, double(maxit), double(damp), Wv, solver, double(tol));
