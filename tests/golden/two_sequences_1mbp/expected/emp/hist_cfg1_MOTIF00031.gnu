set output "hist_cfg1_MOTIF00031.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-53.6478:16.6437]
set yrange [0:2146]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00031.dat" using 1:2 title 'MOTIF00031 (cfg1)' with boxes
