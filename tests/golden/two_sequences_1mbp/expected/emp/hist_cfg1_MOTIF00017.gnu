set output "hist_cfg1_MOTIF00017.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-91.5308:26.3759]
set yrange [0:2824]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00017.dat" using 1:2 title 'MOTIF00017 (cfg1)' with boxes
