% damp = obj.discrep(data, stddev): Tikhonov damping from the discrepancy
% principle (discrep.m:2-69 of the reference).
%
%  data    complex [M nc] or [nr ny nc]
%  stddev  noise standard deviation (guessed from the data if omitted)
%
% 20 updates damp <- damp * discrepancy / norm(A x - data), each solving
% (A'DA + damp^2 I) x = A'D data by MINRES (tol 1e-4, MATLAB's default of 20
% iterations) on the GPU, warm-started from the previous x as the reference
% does with minres(A, b, 1e-4, [], [], [], x).
function damp = discrep(obj, data, stddev)
[nc, ~, ~] = obj.raw_shape(data);
data = reshape(data, obj.M, nc);
if nargin > 2
    validateattributes(stddev, {'numeric'}, {'scalar', 'finite', 'nonnegative'}, '', 'stddev');
else
    tmp = nonzeros(data);
    tmp = [real(tmp); imag(tmp)];
    stddev = median(abs(tmp - median(tmp)));
    warning('stddev not supplied. Guessing %.2e.', stddev);
end
discrepancy = stddev * sqrt(numel(data));
raw = single(data);
if isreal(raw), raw = complex(raw); end
x = complex(zeros([obj.N nc], 'single'));
damp = 0.1;
for iter = 1:20
    if iter == 1
        x = nufft3d_mex('inverse', obj.plan, raw, 20, double(damp), [], 'minres', 1e-4);
    else
        x = nufft3d_mex('inverse_x0', obj.plan, raw, x, 20, double(damp), [], 'minres', 1e-4);
    end
    resnorm = norm(reshape(double(obj.fNUFT(x)) - double(data), [], 1));
    damp = damp * (discrepancy / resnorm);
end
